"""ctypes wrapper around ``refpath.c`` (the C restatement of the reference's own
multiply path). Test infrastructure and CPU baseline only.

``build()`` compiles ``librefpath.so`` beside this file with the committed
Makefile (gcc -O3 -fopenmp). Nothing here reads the reference tree.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import List, Optional, Sequence

import numpy as np

from . import ring

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "librefpath.so")
_lib = None

_u64p = ctypes.POINTER(ctypes.c_uint64)


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "refpath.c")):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "librefpath.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.rp_s_mul.restype = ctypes.c_uint64
        L.rp_s_mul.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.rp_s_mul_device_formula.restype = ctypes.c_uint64
        L.rp_s_mul_device_formula.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.rp_omega.restype = ctypes.c_uint64
        L.rp_omega.argtypes = [ctypes.c_int]
        L.rp_twiddles.restype = None
        L.rp_twiddles.argtypes = [ctypes.c_int, _u64p, _u64p]
        L.rp_mod1_low.restype = ctypes.c_uint64
        L.rp_mod1_low.argtypes = [_u64p, ctypes.c_int, ctypes.c_uint32]
        L.rp_bucket.restype = None
        L.rp_bucket.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int]
        L.rp_create.restype = ctypes.c_void_p
        L.rp_create.argtypes = [_u64p, ctypes.c_int, ctypes.c_int]
        L.rp_destroy.restype = None
        L.rp_destroy.argtypes = [ctypes.c_void_p]
        L.rp_nprimes.restype = ctypes.c_int
        L.rp_nprimes.argtypes = [ctypes.c_void_p]
        L.rp_mwords.restype = ctypes.c_int
        L.rp_mwords.argtypes = [ctypes.c_void_p]
        L.rp_primes.restype = None
        L.rp_primes.argtypes = [ctypes.c_void_p, _u64p]
        L.rp_mul_plain.restype = ctypes.c_int
        L.rp_mul_plain.argtypes = [ctypes.c_void_p, _u64p, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_int,
                                   ctypes.c_int, _u64p]
        L.rp_polymul.restype = ctypes.c_int
        L.rp_polymul.argtypes = [ctypes.c_void_p, _u64p, _u64p, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_int]
        L.rp_yashe_mul.restype = ctypes.c_int
        L.rp_yashe_mul.argtypes = [ctypes.c_void_p, _u64p, _u64p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                   _u64p, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def bucket(count: int = 100) -> List[int]:
    out = (ctypes.c_uint32 * count)()
    lib().rp_bucket(out, count)
    return list(out)


def omega(n: int) -> int:
    return int(lib().rp_omega(n))


def twiddles(n: int):
    W = np.zeros(n, dtype=np.uint64)
    WI = np.zeros(n, dtype=np.uint64)
    lib().rp_twiddles(n, _ptr(W), _ptr(WI))
    return [int(x) for x in W], [int(x) for x in WI]


def mod1_low(words: Sequence[int], p: int) -> int:
    a = np.array(list(words), dtype=np.uint64)
    return int(lib().rp_mod1_low(_ptr(a), len(words), p))


class RefPath:
    """The reference multiply for a fixed q and ``degree`` (gen_crt_primes(q, degree))."""

    def __init__(self, q: int, degree: int):
        self.q = q
        self.qw = ring.nlimbs64(q)
        qa = ring.to_limbs([q], self.qw).reshape(-1)
        self._qa = qa
        self.h = lib().rp_create(_ptr(qa), self.qw, degree)
        self.k = lib().rp_nprimes(self.h)
        self.mw = lib().rp_mwords(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().rp_destroy(self.h)
            self.h = None

    def primes(self) -> List[int]:
        out = np.zeros(self.k, dtype=np.uint64)
        lib().rp_primes(self.h, _ptr(out))
        return [int(x) for x in out]

    def mul_plain(self, a: Sequence[int], b: Sequence[int]) -> List[int]:
        """``Polynomial c = a*b`` (no reduce): coefficients of the product mod M."""
        la = max(1, (max(int(x).bit_length() for x in a) + 63) // 64)
        lb = max(1, (max(int(x).bit_length() for x in b) + 63) // 64)
        A = ring.to_limbs(a, la)
        B = ring.to_limbs(b, lb)
        n = 2
        while n < (len(a) - 1) + (len(b) - 1):
            n <<= 1
        out = np.zeros((n, self.mw), dtype=np.uint64)
        lib().rp_mul_plain(self.h, _ptr(A), len(a), la, _ptr(B), len(b), lb, _ptr(out))
        vals = ring.from_limbs(out)
        return vals[: len(a) + len(b) - 1]

    def polymul(self, a: np.ndarray, b: np.ndarray, nthreads: int = 1) -> np.ndarray:
        """``c = a*b; c.reduce()`` on limb arrays [batch][N][qw] (uint64)."""
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        batch, n = a.shape[0], a.shape[1]
        out = np.zeros_like(a)
        lib().rp_polymul(self.h, _ptr(a), _ptr(b), n, batch, _ptr(out), nthreads)
        return out

    def yashe_mul(self, c1: np.ndarray, c2: np.ndarray, t: int, w_bits: int,
                  evk: Optional[np.ndarray], nthreads: int = 1) -> np.ndarray:
        c1 = np.ascontiguousarray(c1, dtype=np.uint64)
        c2 = np.ascontiguousarray(c2, dtype=np.uint64)
        batch, n = c1.shape[0], c1.shape[1]
        out = np.zeros_like(c1)
        if evk is not None:
            evk = np.ascontiguousarray(evk, dtype=np.uint64)
            ell = evk.shape[0]
            ep = _ptr(evk)
        else:
            ell, ep = 0, None
        lib().rp_yashe_mul(self.h, _ptr(c1), _ptr(c2), n, t, w_bits, ep, ell, batch, _ptr(out), nthreads)
        return out


def s_mul(a: int, b: int) -> int:
    return int(lib().rp_s_mul(a, b))


def s_mul_device_formula(a: int, b: int) -> int:
    return int(lib().rp_s_mul_device_formula(a, b))
