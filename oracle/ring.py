"""Exact arithmetic in Z_q[x]/(x^N+1) with Python integers (test infrastructure).

The reference multiplies two polynomials over Z (CRT + NTT, ``src/common.h:136-226``)
and then ``Polynomial::reduce`` (``src/cuda_functions.cu:1040-1077``) folds the
product by phi = x^N + 1 (``c_i -= c_{i+N}``, lines 1069-1072) and reduces every
coefficient with NTL's ``%= q`` (line 1076, non-negative remainder). phi is built
by ``Polynomial::BuildNthCyclotomic`` (``src/polynomial.cpp:463-469``) as x^N + 1
for a power-of-two N. The functions here restate exactly that result.

Three independent ways to get the product are provided:

* ``plain_mul_schoolbook``: O(N^2) Python loops, for small N only;
* ``plain_mul``: Kronecker substitution, i.e. pack each polynomial into one big
  integer with wide slots, multiply the two integers, unpack signed slots;
* ``NttModQ``: a negacyclic NTT directly modulo q, usable when q = 1 (mod 2N).

The tests cross-check them against each other and against the golden vectors
extracted from the reference's own tests.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np


# ----------------------------------------------------------------------------
# limb layout helpers: [N][L] little-endian uint64 limbs per coefficient
# ----------------------------------------------------------------------------

def nlimbs64(q: int) -> int:
    """64-bit limbs needed to hold values in [0, q)."""
    return max(1, ((q - 1).bit_length() + 63) // 64)


def to_limbs(values: Sequence[int], L: int) -> np.ndarray:
    """Non-negative ints -> uint64 array of shape [len(values), L]."""
    n = len(values)
    raw = b"".join(int(v).to_bytes(8 * L, "little") for v in values)
    return np.frombuffer(raw, dtype="<u8").reshape(n, L).copy()


def from_limbs(arr: np.ndarray) -> List[int]:
    """uint64 array [..., N, L] -> list of Python ints (last axis = limbs)."""
    a = np.ascontiguousarray(arr, dtype="<u8")
    L = a.shape[-1]
    flat = a.reshape(-1, L)
    raw = flat.tobytes()
    w = 8 * L
    return [int.from_bytes(raw[i * w:(i + 1) * w], "little") for i in range(flat.shape[0])]


def centered(x: int, q: int) -> int:
    """Symmetric representative of x mod q in (-q/2, q/2]."""
    x %= q
    return x - q if x > q // 2 else x


# ----------------------------------------------------------------------------
# products over Z
# ----------------------------------------------------------------------------

def plain_mul_schoolbook(a: Sequence[int], b: Sequence[int]) -> List[int]:
    """Full product over Z (length len(a)+len(b)-1). Pure Python, small sizes."""
    if not a or not b:
        return []
    c = [0] * (len(a) + len(b) - 1)
    for i, ai in enumerate(a):
        if ai == 0:
            continue
        for j, bj in enumerate(b):
            c[i + j] += ai * bj
    return c


def _pack(vals: Sequence[int], slot_bytes: int) -> int:
    pos = b"".join(max(v, 0).to_bytes(slot_bytes, "little") for v in vals)
    neg = b"".join(max(-v, 0).to_bytes(slot_bytes, "little") for v in vals)
    return int.from_bytes(pos, "little") - int.from_bytes(neg, "little")


def plain_mul(a: Sequence[int], b: Sequence[int]) -> List[int]:
    """Full product over Z by Kronecker substitution (signed coefficients allowed)."""
    if not a or not b:
        return []
    n_out = len(a) + len(b) - 1
    ma = max(abs(int(v)) for v in a)
    mb = max(abs(int(v)) for v in b)
    if ma == 0 or mb == 0:  # the slot width below is sized from a nonzero product
        return [0] * n_out
    bound = ma * mb * min(len(a), len(b))  # |c_k| <= bound, and >= every input
    slot_bits = bound.bit_length() + 2
    slot_bytes = (slot_bits + 7) // 8
    slot_bits = 8 * slot_bytes
    A = _pack([int(v) for v in a], slot_bytes)
    B = _pack([int(v) for v in b], slot_bytes)
    C = A * B
    # offset every slot by 2^(slot_bits-1) so that each digit is non-negative
    half = 1 << (slot_bits - 1)
    offset = int.from_bytes(half.to_bytes(slot_bytes, "little") * n_out, "little")
    raw = (C + offset).to_bytes(slot_bytes * n_out + 1, "little", signed=False)
    out = []
    for k in range(n_out):
        d = int.from_bytes(raw[k * slot_bytes:(k + 1) * slot_bytes], "little")
        out.append(d - half)
    return out


def fold_negacyclic(c: Sequence[int], n: int) -> List[int]:
    """Reduce a polynomial over Z modulo x^n + 1 (reference ``reduce``, fold step)."""
    out = [0] * n
    for i, v in enumerate(c):
        if (i // n) % 2 == 0:
            out[i % n] += v
        else:
            out[i % n] -= v
    return out


def negacyclic_mul_z(a: Sequence[int], b: Sequence[int]) -> List[int]:
    """a*b over Z[x]/(x^N+1), N = len(a) = len(b)."""
    assert len(a) == len(b)
    return fold_negacyclic(plain_mul(a, b), len(a))


def polymul_mod(a: Sequence[int], b: Sequence[int], q: int) -> List[int]:
    """``Polynomial c = a*b; c.reduce();`` -> coefficients in [0, q).

    Restates ``src/cuda_functions.cu:1061-1076``: fold, then NTL ``% q`` which
    returns the non-negative remainder.
    """
    return [v % q for v in negacyclic_mul_z(a, b)]


def polyadd_mod(a: Sequence[int], b: Sequence[int], q: int) -> List[int]:
    return [(x + y) % q for x, y in zip(a, b)]


# ----------------------------------------------------------------------------
# primes / NTT modulo q (used by the YASHE oracle for keygen when q = 1 mod 2N)
# ----------------------------------------------------------------------------

_MR_BASES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53)


def is_probable_prime(n: int) -> bool:
    if n < 2:
        return False
    for p in _MR_BASES:
        if n % p == 0:
            return n == p
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in _MR_BASES:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def primitive_root_of_unity(order: int, q: int) -> int:
    """An element of exact multiplicative order ``order`` (a power of two) mod q."""
    assert (q - 1) % order == 0 and order & (order - 1) == 0
    for g in range(2, 10_000):
        w = pow(g, (q - 1) // order, q)
        if pow(w, order // 2, q) == q - 1:
            return w
    raise ValueError("no root found")


class NttModQ:
    """Negacyclic NTT modulo a prime q with q = 1 (mod 2N). Pure Python.

    Uses psi (a primitive 2N-th root): NTT(a)_j = sum_i a_i psi^((2j+1) i).
    """

    def __init__(self, n: int, q: int):
        assert (q - 1) % (2 * n) == 0
        self.n, self.q = n, q
        self.psi = primitive_root_of_unity(2 * n, q)
        self.omega = self.psi * self.psi % q
        self.n_inv = pow(n, q - 2, q)
        self.psi_pows = [pow(self.psi, i, q) for i in range(n)]
        self.psi_inv_pows = [pow(pow(self.psi, q - 2, q), i, q) for i in range(n)]

    def _cyclic(self, a: List[int], w: int) -> List[int]:
        n, q = len(a), self.q
        a = list(a)
        # iterative radix-2, bit reversal first
        j = 0
        for i in range(1, n):
            bit = n >> 1
            while j & bit:
                j ^= bit
                bit >>= 1
            j |= bit
            if i < j:
                a[i], a[j] = a[j], a[i]
        length = 2
        while length <= n:
            wl = pow(w, n // length, q)
            half = length // 2
            ws = [1] * half
            for k in range(1, half):
                ws[k] = ws[k - 1] * wl % q
            for s in range(0, n, length):
                for k in range(half):
                    u = a[s + k]
                    v = a[s + k + half] * ws[k] % q
                    a[s + k] = (u + v) % q
                    a[s + k + half] = (u - v) % q
            length <<= 1
        return a

    def forward(self, a: Sequence[int]) -> List[int]:
        q = self.q
        return self._cyclic([x * p % q for x, p in zip(a, self.psi_pows)], self.omega)

    def inverse(self, A: Sequence[int]) -> List[int]:
        q = self.q
        a = self._cyclic(list(A), pow(self.omega, q - 2, q))
        return [x * self.n_inv % q * p % q for x, p in zip(a, self.psi_inv_pows)]

    def mul(self, a: Sequence[int], b: Sequence[int]) -> List[int]:
        q = self.q
        A, B = self.forward(a), self.forward(b)
        return self.inverse([x * y % q for x, y in zip(A, B)])


def poly_inverse_mod(f: Sequence[int], q: int) -> List[int]:
    """f^-1 in Z_q[x]/(x^N+1) for prime q.

    q = 1 (mod 2N): pointwise inversion in the NTT domain. Otherwise the extended
    Euclidean algorithm over F_q[x] (quadratic, meant for small N).
    Raises ValueError when f is not invertible.
    """
    n = len(f)
    if (q - 1) % (2 * n) == 0:
        ntt = NttModQ(n, q)
        F = ntt.forward([x % q for x in f])
        if any(v == 0 for v in F):
            raise ValueError("f is not invertible")
        return ntt.inverse([pow(v, q - 2, q) for v in F])
    return _poly_inverse_euclid(f, q)


def _trim(p: List[int]) -> List[int]:
    while p and p[-1] == 0:
        p.pop()
    return p


def _poly_inverse_euclid(f: Sequence[int], q: int) -> List[int]:
    n = len(f)
    r0 = [1] + [0] * (n - 1) + [1]  # x^n + 1
    r1 = _trim([x % q for x in f])
    s0, s1 = [], [1]
    while len(r1) > 1:
        # r0 = quo * r1 + rem
        rem = list(r0)
        quo = [0] * (len(r0) - len(r1) + 1)
        inv_lead = pow(r1[-1], q - 2, q)
        while len(_trim(rem)) >= len(r1):
            d = len(rem) - len(r1)
            coef = rem[-1] * inv_lead % q
            quo[d] = coef
            for i, v in enumerate(r1):
                rem[d + i] = (rem[d + i] - coef * v) % q
            _trim(rem)
        # s_new = s0 - quo * s1
        prod = plain_mul_schoolbook(quo, s1) if s1 and quo else []
        m = max(len(s0), len(prod))
        s_new = [((s0[i] if i < len(s0) else 0) - (prod[i] if i < len(prod) else 0)) % q for i in range(m)]
        r0, r1 = r1, _trim(rem)
        s0, s1 = s1, _trim(s_new)
    if not r1:
        raise ValueError("f is not invertible")
    c = pow(r1[0], q - 2, q)
    inv = [(v * c) % q for v in s1] + [0] * n
    return inv[:n]


def largest_prime_below(bound: int, congruent_mod: int = 1) -> int:
    """Largest prime p < bound with p = 1 (mod congruent_mod)."""
    p = ((bound - 2) // congruent_mod) * congruent_mod + 1
    while not is_probable_prime(p):
        p -= congruent_mod
    return p


def primes_below_descending(bound: int, count: int) -> List[int]:
    """The ``count`` largest primes below ``bound``, descending.

    With bound = 2^29 and count = 100 this regenerates the reference's
    ``PRIMES_BUCKET`` (``src/polynomial.cpp:22``); the golden fixture pins it.
    """
    out, n = [], bound - 1
    while len(out) < count:
        if is_probable_prime(n):
            out.append(n)
        n -= 1
    return out
