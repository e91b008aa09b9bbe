"""Host-buffer entry points (cy_polymul_host, cy_yashe_mul_host): a batch runs in
chunks whose host<->device copies overlap the kernels of neighbouring chunks.

Every result must equal the device-buffer call's bit for bit, for pageable
(numpy) and page-locked (pinned torch) buffers, for batches of one chunk, of
several chunks and with a ragged last chunk; a few products are also checked
against the oracle.
"""
import random

import numpy as np
import pytest

from oracle import ring
from oracle.yashe import Yashe as OYashe
from oracle.yashe import YasheParams

pytestmark = pytest.mark.gpu

INVALID, NO_KEYS = -1, -6  # cy_status codes (include/cuyashe.h)
Q127 = 2**127 - 1
QY = 170141183460469231731687303715883253761  # largest prime < 2^127 with q = 1 mod 2^16


@pytest.fixture(scope="module")
def cy():
    import torch

    import cuyashe_gb300

    assert torch.cuda.is_available()
    cuyashe_gb300.lib()
    return cuyashe_gb300


def _rand_words(rng, shape, top_bits):
    x = rng.integers(0, 2**64, size=shape, dtype=np.uint64)
    x[..., -1] &= np.uint64((1 << top_bits) - 1)
    return x


@pytest.mark.parametrize("batch", [1, 170, 700])  # one chunk (24 MiB of residues), several, ragged
def test_polymul_host_matches_device(cy, batch):
    import torch

    R = cy.Ring(4096, Q127)
    rng = np.random.default_rng(batch)
    a = _rand_words(rng, (batch, 4096, 2), 62)
    b = _rand_words(rng, (batch, 4096, 2), 62)
    dev = R.polymul(torch.from_numpy(a.view(np.int64)).cuda(), torch.from_numpy(b.view(np.int64)).cuda())
    want = dev.cpu().numpy().view(np.uint64)
    got = R.polymul_host(a, b)                      # pageable
    assert np.array_equal(got, want)
    pa = torch.from_numpy(a.view(np.int64)).pin_memory()
    pb = torch.from_numpy(b.view(np.int64)).pin_memory()
    po = torch.empty_like(pa).pin_memory()
    R.polymul_host(pa, pb, out=po)                  # page-locked
    assert np.array_equal(po.numpy().view(np.uint64), want)


def test_polymul_host_matches_oracle_across_chunks(cy):
    # N = 1024 with k = 9 primes: 682 products per 24 MiB chunk, so 1000 is two chunks
    n, batch = 1024, 1000
    R = cy.Ring(n, Q127)
    rng = np.random.default_rng(3)
    a = _rand_words(rng, (batch, n, 2), 62)
    b = _rand_words(rng, (batch, n, 2), 62)
    got = R.polymul_host(a, b)
    for j in (0, 681, 682, 999):
        A = [int(a[j, i, 0]) | (int(a[j, i, 1]) << 64) for i in range(n)]
        B = [int(b[j, i, 0]) | (int(b[j, i, 1]) << 64) for i in range(n)]
        C = [int(got[j, i, 0]) | (int(got[j, i, 1]) << 64) for i in range(n)]
        assert C == ring.polymul_mod(A, B, Q127)


@pytest.mark.parametrize("relin", [True, False])
def test_yashe_mul_host_matches_device(cy, relin):
    import torch

    n, t, batch = 4096, 1024, 500
    Y = cy.Yashe(n, QY, t)
    Y.keygen(11)
    rng = np.random.default_rng(5)
    m = rng.integers(0, t, size=(2 * 8, n), dtype=np.uint64)
    ct = Y.encrypt_host(m, seed=9)
    idx = np.arange(batch)
    c1 = np.ascontiguousarray(ct[idx % 8])
    c2 = np.ascontiguousarray(ct[8 + (idx * 3) % 8])
    d1 = torch.from_numpy(c1.view(np.int64)).cuda()
    d2 = torch.from_numpy(c2.view(np.int64)).cuda()
    want = Y.mul(d1, d2, relin=relin).cpu().numpy().view(np.uint64)
    assert np.array_equal(Y.mul_host(c1, c2, relin=relin), want)
    p1 = torch.from_numpy(c1.view(np.int64)).pin_memory()
    p2 = torch.from_numpy(c2.view(np.int64)).pin_memory()
    po = torch.empty_like(p1).pin_memory()
    Y.mul_host(p1, p2, out=po, relin=relin)
    assert np.array_equal(po.numpy().view(np.uint64), want)


def test_yashe_mul_host_matches_oracle(cy):
    n, t = 64, 257
    q = ring.largest_prime_below(2**127, congruent_mod=2 * n)
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    keys = oy.keygen(21)
    rng = random.Random(2)
    pts = [[rng.randrange(t) for _ in range(n)] for _ in range(4)]
    cts = [oy.encrypt(keys, m, 100 + i) for i, m in enumerate(pts)]
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    L = Y.ring.L
    h = np.array([[[(v >> (64 * w)) & (2**64 - 1) for w in range(L)] for v in c] for c in cts], dtype=np.uint64)
    out = Y.mul_host(h[:2], h[2:], relin=True)
    for j in range(2):
        got = [sum(int(out[j, i, w]) << (64 * w) for w in range(L)) for i in range(n)]
        assert got == oy.mul(keys, cts[j], cts[2 + j], relin=True)
        assert oy.decrypt(keys, got) == ring.polymul_mod(pts[j], pts[2 + j], t)


def test_host_entry_points_reject_bad_arguments(cy):
    R = cy.Ring(1024, Q127)
    Y = cy.Yashe(1024, QY, 1024)
    buf = np.zeros((1, 1024, 2), np.uint64)
    lib = cy.lib()
    assert lib.cy_polymul_host(R.h, 0, buf.ctypes.data, buf.ctypes.data, 1) == INVALID
    assert lib.cy_yashe_mul_host(Y.h, buf.ctypes.data, buf.ctypes.data, 0, 1, 0) == INVALID
    assert lib.cy_yashe_mul_host(Y.h, buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 1, 1) == NO_KEYS
    assert lib.cy_yashe_mul_host(Y.h, buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 0, 0) == 0
    assert lib.cy_yashe_mul_host(None, buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 1, 0) != 0


def test_chunk_overlap_gives_identical_results(cy):
    """Several chunks run on two streams by default; serial chunks must give the
    same products and HE multiplies bit for bit."""
    import torch

    n, t, batch = 4096, 1024, 700  # 170 tensor products per chunk: five chunks
    Y = cy.Yashe(n, QY, t)
    Y.keygen(3)
    rng = np.random.default_rng(9)
    m = torch.from_numpy(rng.integers(0, t, size=(batch, n), dtype=np.uint64).view(np.int64)).cuda()
    c1, c2 = Y.encrypt(m, seed=1), Y.encrypt(m.flip(0).contiguous(), seed=2)
    R = cy.Ring(n, Q127)
    a = torch.from_numpy(_rand_words(rng, (batch, n, 2), 62).view(np.int64)).cuda()
    b = torch.from_numpy(_rand_words(rng, (batch, n, 2), 62).view(np.int64)).cuda()
    lib = cy.lib()
    outs = []
    for overlap in (1, 0):
        lib.cy_set_chunk_overlap(overlap)
        try:
            outs.append((Y.mul(c1, c2, relin=True), R.polymul(a, b)))
            torch.cuda.synchronize()
        finally:
            lib.cy_set_chunk_overlap(1)
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
