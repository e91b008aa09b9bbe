"""The counter-based Gaussian sampler of the GPU encryption, on the CPU.

The oracle's restatement (oracle/sampling.py) must equal a sequential
splitmix64 stream, give a discrete Gaussian of the stated width, and build the
same CDT thresholds as the library (cy_gaussian_cdt, a host-only entry point).
"""
import ctypes

import numpy as np
import pytest

from oracle import sampling


def test_counter_draws_equal_the_sequential_stream():
    for seed in (0, 1, 0xDEADBEEF, 2**64 - 1):
        seq = sampling.splitmix64_sequence(seed, 300)
        ctr = sampling.counter_draws(seed, np.arange(300, dtype=np.uint64))
        assert [int(v) for v in ctr] == seq


@pytest.mark.parametrize("sigma", [3.2, 8.0, 19.2])
def test_cdt_is_a_discrete_gaussian(sigma):
    T = sampling.gaussian_cdt(sigma)
    B = (len(T) - 1) // 2
    assert B == int(np.ceil(6 * sigma))
    assert all(a <= b for a, b in zip(T, T[1:])) and T[-1] == 2**64 - 1
    x = sampling.gaussian_from_draws(T, sampling.counter_draws(7, np.arange(400_000, dtype=np.uint64)))
    assert x.min() >= -B and x.max() <= B
    assert abs(x.mean()) < 0.05 * sigma
    assert abs(x.std() / sigma - 1.0) < 0.02
    # symmetric tails
    assert abs((x > sigma).mean() - (x < -sigma).mean()) < 0.01


def test_edges_of_the_threshold_map():
    T = sampling.gaussian_cdt(8.0)
    B = (len(T) - 1) // 2
    d = np.array([0, T[0] - 1, T[0], T[B] - 1, T[B], 2**64 - 2, 2**64 - 1], dtype=np.uint64)
    x = sampling.gaussian_from_draws(T, d)
    assert list(x[:3]) == [-B, -B, -B + 1]
    assert list(x[3:5]) == [0, 1]
    assert x[-1] == B and x[-2] == B


@pytest.mark.parametrize("sigma", [3.2, 8.0, 19.2])
def test_library_builds_the_same_thresholds(sigma):
    import cuyashe_gb300 as cy

    lib = cy.lib()
    buf = (ctypes.c_uint64 * 1024)()
    n = ctypes.c_int(0)
    assert lib.cy_gaussian_cdt(sigma, buf, 1024, ctypes.byref(n)) == 0
    assert list(buf[: n.value]) == sampling.gaussian_cdt(sigma)
    small = (ctypes.c_uint64 * 4)()
    assert lib.cy_gaussian_cdt(sigma, small, 4, ctypes.byref(n)) != 0 and n.value == len(sampling.gaussian_cdt(sigma))
    assert lib.cy_gaussian_cdt(-1.0, buf, 1024, ctypes.byref(n)) != 0


def test_encryption_errors_layout():
    s, e = sampling.encryption_errors(5, 3, 16, 8.0)
    T = sampling.gaussian_cdt(8.0)
    for b in range(3):
        for i in range(16):
            ds = sampling.counter_draws(5, np.array([2 * b * 16 + i], dtype=np.uint64))
            de = sampling.counter_draws(5, np.array([(2 * b + 1) * 16 + i], dtype=np.uint64))
            assert s[b, i] == sampling.gaussian_from_draws(T, ds)[0]
            assert e[b, i] == sampling.gaussian_from_draws(T, de)[0]
