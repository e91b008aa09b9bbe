"""YASHE oracle (test infrastructure): Bos, Lauter, Loftus, Naehrig, "Improved
security for a ring-based fully homomorphic encryption scheme" (IMA CC 2013).

The reference implements the scheme in ``src/yashe.cpp`` and
``src/ciphertext.cpp``. This restatement follows the formulas it intends and
corrects the defects that the reference's own code has when read:

* keygen (``src/yashe.cpp:17-102``): f = t*f' + 1 with ternary f'; the reference
  replaces f^-1 by f (lines 48-50); here f^-1 is a real inverse in R_q.
  h = [t * g * f^-1]_q; evaluation key gamma_d = [f * w^d + e_d + h * s_d]_q
  (lines 70-93) for d = 0..ell-1 with w = 2^w_bits.
* encrypt (``src/yashe.cpp:104-142``): c = [h*s + e + Delta*m]_q, Delta = floor(q/t).
* multiply (``src/ciphertext.cpp:38-73``): c = [round(t/q * c1*c2)]_q where the
  product is taken over Z[x]/(x^N+1) on the symmetric representatives of c1 and
  c2. The reference multiplies by t after an in-place op whose result is dropped
  and reduces mod q before dividing; both are corrected here.
* relinearisation (``src/ciphertext.cpp:75-130``): c' = [sum_d D_d(c) * gamma_d]_q
  with D_d(c) the base-2^w_bits digits of c in [0, q) (the reference's mask is a
  single bit and its digit polynomials are copies, both corrected).
* decrypt (``src/yashe.cpp:143-201``): m = [round(t/q * [f*c]_q)]_t for every
  coefficient (the reference decrypts coefficient 0 only); ciphertexts that come
  out of a multiply without relinearisation decrypt with f^2 (lines 154-158).

Sampling uses numpy's PCG64 with an explicit seed; the error distribution is a
discrete Gaussian of parameter sigma truncated at 6*sigma, sampled from its CDT.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import ring


@dataclass
class YasheParams:
    n: int
    q: int
    t: int
    w_bits: int = 32
    sigma: float = 8.0

    @property
    def delta(self) -> int:
        return self.q // self.t

    @property
    def ell(self) -> int:
        """Number of base-2^w_bits digits of a value in [0, q)."""
        return -(-(self.q - 1).bit_length() // self.w_bits)


@dataclass
class YasheKeys:
    f: List[int]
    h: List[int]
    evk: List[List[int]]
    f2: List[int] = field(default_factory=list)


class Sampler:
    def __init__(self, seed: int):
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self._cdt_cache = {}

    def ternary(self, n: int) -> List[int]:
        return [int(v) for v in self.rng.integers(-1, 2, size=n)]

    def gaussian(self, n: int, sigma: float) -> List[int]:
        bound = int(math.ceil(6 * sigma))
        if sigma not in self._cdt_cache:
            xs = np.arange(-bound, bound + 1)
            w = np.exp(-(xs.astype(np.float64) ** 2) / (2.0 * sigma * sigma))
            self._cdt_cache[sigma] = (xs, w / w.sum())
        xs, p = self._cdt_cache[sigma]
        return [int(v) for v in self.rng.choice(xs, size=n, p=p)]

    def uniform(self, n: int, modulus: int) -> List[int]:
        nbits = max(1, (modulus - 1).bit_length())
        nwords = (nbits + 63) // 64
        out = []
        while len(out) < n:
            words = self.rng.integers(0, 2**64, size=nwords, dtype=np.uint64)
            v = 0
            for i, wd in enumerate(words):
                v |= int(wd) << (64 * i)
            v &= (1 << nbits) - 1
            if v < modulus:
                out.append(v)
        return out


def _mul_mod_q(a: Sequence[int], b: Sequence[int], q: int, ntt: Optional[ring.NttModQ]) -> List[int]:
    if ntt is not None:
        return ntt.mul([x % q for x in a], [x % q for x in b])
    return ring.polymul_mod(a, b, q)


class Yashe:
    """The YASHE scheme over R_q = Z_q[x]/(x^N+1)."""

    def __init__(self, params: YasheParams):
        self.p = params
        n, q = params.n, params.q
        self._ntt = ring.NttModQ(n, q) if (q - 1) % (2 * n) == 0 else None

    # -- key generation ---------------------------------------------------
    def keygen(self, seed: int) -> YasheKeys:
        p = self.p
        n, q, t = p.n, p.q, p.t
        smp = Sampler(seed)
        g = smp.ternary(n)
        while True:
            fp = smp.ternary(n)
            f = [(t * v) % q for v in fp]
            f[0] = (f[0] + 1) % q
            try:
                f_inv = ring.poly_inverse_mod(f, q)
                break
            except ValueError:
                continue
        tg = [(t * v) % q for v in g]
        h = _mul_mod_q(tg, f_inv, q, self._ntt)
        evk = []
        for d in range(p.ell):
            wd = pow(2, p.w_bits * d, q)
            e = smp.gaussian(n, p.sigma)
            s = smp.gaussian(n, p.sigma)
            hs = _mul_mod_q(h, s, q, self._ntt)
            evk.append([(fv * wd + ev + hv) % q for fv, ev, hv in zip(f, e, hs)])
        f2 = _mul_mod_q(f, f, q, self._ntt)
        return YasheKeys(f=f, h=h, evk=evk, f2=f2)

    # -- encryption / decryption ------------------------------------------
    def encrypt(self, keys: YasheKeys, m: Sequence[int], seed: int) -> List[int]:
        p = self.p
        smp = Sampler(seed)
        s = smp.gaussian(p.n, p.sigma)
        e = smp.gaussian(p.n, p.sigma)
        hs = _mul_mod_q(keys.h, s, p.q, self._ntt)
        dm = [(p.delta * (mv % p.t)) for mv in m]
        return [(hv + ev + dv) % p.q for hv, ev, dv in zip(hs, e, dm)]

    def encrypt_with_errors(self, keys: YasheKeys, m: Sequence[int], s: Sequence[int],
                            e: Sequence[int]) -> List[int]:
        """[h*s + e + Delta*(m mod t)]_q for given error polynomials s, e
        (the formula of encrypt above; the GPU encryption draws s and e with
        the counter-based sampler of oracle/sampling.py)."""
        p = self.p
        hs = _mul_mod_q(keys.h, [int(v) for v in s], p.q, self._ntt)
        return [(hv + int(ev) + p.delta * (int(mv) % p.t)) % p.q for hv, ev, mv in zip(hs, e, m)]

    def add_plain(self, c: Sequence[int], m: Sequence[int]) -> List[int]:
        """[c + Delta*(m mod t)]_q (a plaintext added to a ciphertext)."""
        p = self.p
        return [(int(cv) + p.delta * (int(mv) % p.t)) % p.q for cv, mv in zip(c, m)]

    def mul_plain(self, c: Sequence[int], m: Sequence[int]) -> List[int]:
        """[c * m_c]_q with m_c the representative of m mod t in (-t/2, t/2]."""
        p = self.p
        mc = [(int(mv) % p.t) - (p.t if (int(mv) % p.t) > p.t // 2 else 0) for mv in m]
        return _mul_mod_q(list(c), mc, p.q, self._ntt)

    def decrypt(self, keys: YasheKeys, c: Sequence[int], aftermul: bool = False) -> List[int]:
        p = self.p
        key = keys.f2 if aftermul else keys.f
        x = _mul_mod_q(key, c, p.q, self._ntt)
        out = []
        for v in x:
            vc = ring.centered(v, p.q)
            out.append(round_div(p.t * vc, p.q) % p.t)
        return out

    def noise(self, keys: YasheKeys, c: Sequence[int], m: Sequence[int], aftermul: bool = False) -> int:
        """max |[key*c]_q - Delta*m| (centered); decryption is correct while < Delta/2."""
        p = self.p
        key = keys.f2 if aftermul else keys.f
        x = _mul_mod_q(key, c, p.q, self._ntt)
        return max(abs(ring.centered(v - p.delta * (mv % p.t), p.q)) for v, mv in zip(x, m))

    # -- homomorphic operations -------------------------------------------
    def mul_tensor(self, c1: Sequence[int], c2: Sequence[int]) -> List[int]:
        """[round(t/q * c1*c2)]_q with the product over Z[x]/(x^N+1) (no relinearisation)."""
        p = self.p
        a = [ring.centered(v, p.q) for v in c1]
        b = [ring.centered(v, p.q) for v in c2]
        prod = ring.negacyclic_mul_z(a, b)
        return [round_div(p.t * v, p.q) % p.q for v in prod]

    def digits(self, c: Sequence[int]) -> List[List[int]]:
        p = self.p
        mask = (1 << p.w_bits) - 1
        return [[(v >> (p.w_bits * d)) & mask for v in c] for d in range(p.ell)]

    def keyswitch(self, keys: YasheKeys, c: Sequence[int]) -> List[int]:
        """[sum_d D_d(c) * gamma_d]_q."""
        p = self.p
        acc = [0] * p.n
        for dpoly, gamma in zip(self.digits(c), keys.evk):
            prod = _mul_mod_q(dpoly, gamma, p.q, self._ntt)
            acc = [(x + y) % p.q for x, y in zip(acc, prod)]
        return acc

    def mul(self, keys: YasheKeys, c1: Sequence[int], c2: Sequence[int], relin: bool = True) -> List[int]:
        c = self.mul_tensor(c1, c2)
        return self.keyswitch(keys, c) if relin else c

    def add(self, c1: Sequence[int], c2: Sequence[int]) -> List[int]:
        return ring.polyadd_mod(c1, c2, self.p.q)


def round_div(x: int, q: int) -> int:
    """round(x/q) to the nearest integer for odd q > 0 (no ties exist).

    Matches the reference's ``quot = g/q; diff = g%q; if 2*diff > q: quot+1``
    (``src/ciphertext.cpp:55-63``) with NTL's floor division.
    """
    quot, rem = divmod(x, q)
    return quot + 1 if 2 * rem > q else quot
