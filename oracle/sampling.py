"""Counter-based sampling of YASHE's error polynomials (TEST INFRASTRUCTURE ONLY).

This module is part of the oracle: only tests/, the smoke check and the
benchmark's CPU baseline may import it, as a checker; the product never does.

The reference samples its errors with cuRAND uniform draws reduced mod a small
bound (src/cuda_distribution.cu:11-35, src/distribution.cpp:9-51) although the
scheme asks for a discrete Gaussian; its draws are not reproducible outside
cuRAND. The GPU encryption of this project (cy_yashe_encrypt, include/cuyashe.h)
instead specifies its randomness exactly, and this file restates that
specification so that every coefficient the GPU draws can be checked:

* draw c of a call with seed S is the c-th output of splitmix64 seeded with S:
  z = S + (c+1) * 0x9E3779B97F4A7C15, then the splitmix64 finaliser;
* the discrete Gaussian of width sigma on [-B, B], B = ceil(6 sigma), maps a
  draw u to j - B for the first j with u < T[j], T[j] = floor(2^64 * acc_j),
  acc_j the running sum of w_x / sum(w), w_x = exp(-x^2 / (2 sigma^2)),
  accumulated in IEEE double in the order x = -B .. B (T[-1] = 2^64 - 1);
* coefficient i of s (of e) of ciphertext b uses counter 2b*N + i ((2b+1)*N + i).
"""
from __future__ import annotations

import math
from typing import List, Sequence

import numpy as np

GOLDEN = 0x9E3779B97F4A7C15
M64 = (1 << 64) - 1


def splitmix64_sequence(seed: int, count: int) -> List[int]:
    """The first `count` outputs of a sequential splitmix64 (pure Python)."""
    s, out = seed & M64, []
    for _ in range(count):
        s = (s + GOLDEN) & M64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        out.append(z ^ (z >> 31))
    return out


def counter_draws(seed: int, counters: np.ndarray) -> np.ndarray:
    """Draw number c (numpy uint64 array of counters) of a call seeded with `seed`."""
    with np.errstate(over="ignore"):
        c = counters.astype(np.uint64)
        z = np.uint64(seed & M64) + (c + np.uint64(1)) * np.uint64(GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def gaussian_cdt(sigma: float) -> List[int]:
    """64-bit CDT thresholds of D_sigma on [-B, B] (see the module docstring)."""
    bound = int(math.ceil(6.0 * sigma))
    w = []
    total = 0.0
    for j in range(2 * bound + 1):
        x = j - bound
        v = math.exp(-float(x * x) / (2.0 * sigma * sigma))
        w.append(v)
        total += v
    T, acc = [], 0.0
    for v in w:
        acc += v / total
        T.append(M64 if acc >= 1.0 else int(acc * 18446744073709551616.0))
    T[-1] = M64
    return T


def gaussian_from_draws(T: Sequence[int], draws: np.ndarray) -> np.ndarray:
    """Map uint64 draws to samples in [-B, B] with thresholds T."""
    bound = (len(T) - 1) // 2
    idx = np.searchsorted(np.array(T, dtype=np.uint64), draws, side="right")
    return np.minimum(idx, len(T) - 1).astype(np.int64) - bound


def encryption_errors(seed: int, batch: int, n: int, sigma: float):
    """(s, e) of ciphertexts 0 .. batch-1 of one GPU encryption call: int64 [batch][n]."""
    T = gaussian_cdt(sigma)
    b = np.arange(batch, dtype=np.uint64)[:, None]
    i = np.arange(n, dtype=np.uint64)[None, :]
    s = gaussian_from_draws(T, counter_draws(seed, (np.uint64(2) * b) * np.uint64(n) + i))
    e = gaussian_from_draws(T, counter_draws(seed, (np.uint64(2) * b + np.uint64(1)) * np.uint64(n) + i))
    return s, e
