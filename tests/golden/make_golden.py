"""Extract the reference's own known-answer vectors and constants into
``reference_vectors.json``.

Run in the build container, where the reference tree is mounted:

    python tests/golden/make_golden.py /root/reference

It reads the reference's test and source files as text (nothing is compiled or
run) and records, with the file:line each value comes from:

* ``src/test_mul.cu`` second test: explicit a (8 coefficients), b (8 coefficients
  of ~96 bits), q, and the expected plain product over Z (15 coefficients).
* ``src/test.cu``: the PolySuite / YasheSuite parameters (q, degree, t, w, seed).
* ``src/polynomial.cpp``: the PRIMES_BUCKET table of 29-bit CRT primes.
* ``src/cuda_functions.cu``: the Goldilocks prime and its primitive root.
* ``src/test_bnt.cu``: the CRT/ICRT round-trip value and its modulus.
* ``src/benchmark_polynomial.cpp`` / ``src/benchmark_yashe.cpp``: q = 2^127 - 1,
  the benchmark degree and the keyswitch base w.

The JSON is committed; tests only read the JSON.
"""
from __future__ import annotations

import json
import os
import re
import sys


def _line_of(text: str, needle: str) -> int:
    idx = text.index(needle)
    return text.count("\n", 0, idx) + 1


def main(ref_root: str) -> dict:
    src = os.path.join(ref_root, "src")

    def read(name):
        with open(os.path.join(src, name), encoding="utf-8", errors="replace") as fh:
            return fh.read()

    out: dict = {"source": "cuYASHE reference tree, read as text"}

    # --- test_mul.cu, second test --------------------------------------------
    tm = read("test_mul.cu")
    second = tm[tm.index("Second test"):]
    a_vals = {int(i): int(v) for i, v in re.findall(r"a\.set_coeff\((\d+),(\d+)\);", second)}
    b_vals = {int(i): int(v) for i, v in re.findall(r'b\.set_coeff\((\d+),to_ZZ\("(\d+)"\)\);', second)}
    exp2 = re.search(r"ZZ expected_result2\[\] = \{(.*?)\};", second, re.S).group(1)
    expected2 = [int(v) for v in re.findall(r'to_ZZ\("(\d+)"\)', exp2)]
    q_mul = int(re.search(r'global_mod = conv<ZZ>\("(\d+)"\)', tm).group(1))
    deg_mul = int(re.search(r"degree = (\d+);", tm).group(1))
    out["test_mul_2"] = {
        "cite": "src/test_mul.cu:%d-%d" % (_line_of(tm, "Second test"), _line_of(tm, "expected_result2[]")),
        "q": str(q_mul),
        "degree": deg_mul,
        "a": [str(a_vals[i]) for i in range(len(a_vals))],
        "b": [str(b_vals[i]) for i in range(len(b_vals))],
        "expected_plain_product": [str(v) for v in expected2],
    }

    # --- test.cu fixtures ----------------------------------------------------
    tc = read("test.cu")
    qs = re.findall(r'q = conv<ZZ>\("(\d+)L?"\);', tc)
    out["poly_suite"] = {
        "cite": "src/test.cu:%d-%d" % (_line_of(tc, "struct PolySuite"), _line_of(tc, "srand (36251)")),
        "q": str(int(qs[0])),
        "degree": int(re.search(r"PolySuite\(\)\{.*?degree = (\d+);", tc, re.S).group(1)),
        "srand": 36251,
        "ntests": int(re.search(r"#define NTESTS (\d+)", tc).group(1)),
    }
    ys = tc[tc.index("struct YasheSuite"):]
    out["yashe_suite"] = {
        "cite": "src/test.cu:%d" % _line_of(tc, "struct YasheSuite"),
        "q": str(int(re.search(r'q = conv<ZZ>\("(\d+)L?"\);', ys).group(1))),
        "t": int(re.search(r"t = (\d+);", ys).group(1)),
        "degree": int(re.search(r"degree = (\d+);", ys).group(1)),
        "w": int(re.search(r"int w = (\d+);", ys).group(1)),
    }

    # --- PRIMES_BUCKET --------------------------------------------------------
    pc = read("polynomial.cpp")
    bucket = re.search(r"const uint32_t PRIMES_BUCKET\[\] = \{([^}]*)\}", pc).group(1)
    out["primes_bucket"] = {
        "cite": "src/polynomial.cpp:%d" % _line_of(pc, "const uint32_t PRIMES_BUCKET[]"),
        "values": [int(v) for v in bucket.split(",") if v.strip()],
    }

    # --- Goldilocks -----------------------------------------------------------
    cf = read("cuda_functions.cu")
    m_p = re.search(r"^#define PRIMEP \(uint64_t\)(\d+)", cf, re.M)
    m_r = re.search(r"^#define PRIMITIVE_ROOT \(int\)(\d+)\s*$", cf, re.M)
    out["goldilocks"] = {
        "cite": "src/cuda_functions.cu:%d-%d" % (_line_of(cf, m_p.group(0)), _line_of(cf, m_r.group(0))),
        "P": str(int(m_p.group(1))),
        "root": int(m_r.group(1)),
    }

    # --- test_bnt.cu CRT round trip ------------------------------------------
    tb = read("test_bnt.cu")
    x = re.search(r'ZZ X = to_ZZ\("(\d+)"\);', tb)
    qb = re.search(r'gen_crt_primes\(to_ZZ\("(\d+)L?"\),(\d+)\);', tb)
    out["test_bnt_crt"] = {
        "cite": "src/test_bnt.cu:%d-%d" % (_line_of(tb, x.group(0)), _line_of(tb, qb.group(0))),
        "x": x.group(1),
        "q": qb.group(1),
        "degree": int(qb.group(2)),
    }

    # --- benchmark parameters -------------------------------------------------
    bp = read("benchmark_polynomial.cpp")
    by = read("benchmark_yashe.cpp")
    out["benchmark"] = {
        "cite_q": "src/benchmark_polynomial.cpp:%d-%d" % (_line_of(bp, "NTL::power2(q,127);"),
                                                          _line_of(bp, 'q -= conv<ZZ>("1");')),
        "q": str(2**127 - 1),
        "degree": int(re.search(r"^\s*for\(int d = (\d+);d <= 4096", bp, re.M).group(1)),
        "cite_w": "src/benchmark_yashe.cpp:%d" % _line_of(by, "uint64_t w = 4294967296;"),
        "w": 4294967296,
    }
    return out


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    data = main(root)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.json")
    with open(path, "w") as fh:
        json.dump(data, fh, indent=1)
        fh.write("\n")
    print("wrote", path)
