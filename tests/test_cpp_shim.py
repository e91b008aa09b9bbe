"""The C++ API (include/cuyashe.hpp: Polynomial / Ciphertext / Yashe with the
reference's method names) built into the test program tests/cpp/test_shim.cpp,
which mirrors the reference's PolySuite and YasheSuite (src/test.cu).

The CPU test compiles and links the program against the in-tree library; the
GPU test runs it: every case compares GPU results with host big-integer
arithmetic and the program exits with the number of failed cases.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _build_shim_test(out_dir):
    import cuyashe_gb300.build as b

    lib = b.build()
    cuda = _cuda_home()
    exe = os.path.join(str(out_dir), "test_shim")
    cmd = [
        "g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
        "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
        os.path.join(HERE, "cpp", "test_shim.cpp"), "-o", exe,
        "-L" + os.path.dirname(lib), "-lcuyashe_gb300",
        "-L" + os.path.join(cuda, "lib64"), "-lcudart",
        "-Wl,-rpath," + os.path.dirname(lib),
    ]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    return exe


def test_cpp_api_compiles_and_links(tmp_path):
    assert os.path.exists(_build_shim_test(tmp_path))


@pytest.mark.gpu
def test_cpp_api_reference_suites(tmp_path):
    exe = _build_shim_test(tmp_path)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    lines = [l for l in res.stdout.splitlines() if l.startswith(("ok", "FAIL"))]
    assert len(lines) >= 23 and all(l.startswith("ok") for l in lines), res.stdout
