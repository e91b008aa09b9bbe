"""The allocation-free product (cy_polymul_noalloc) against cy_polymul and the oracle.

cy_polymul_noalloc exists for callers that may not call cudaMalloc: serving
paths that cannot take cudaMalloc's device-wide synchronisation, and hosts
whose device memory belongs to another allocator or to a fixed budget. It keeps
its scratch in a fixed array inside the library instead of a workspace. Its
results must equal the ordinary entry point's bit for bit (and the oracle's),
on consecutive calls that reuse the shared array, and batches too large for one
call must be refused with a clear message.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes when run alone.
"""
import random

import pytest

from oracle import ring

pytestmark = pytest.mark.gpu

NOALLOC_SCRATCH_BYTES = 16 << 20  # CY_NOALLOC_SCRATCH_BYTES in include/cuyashe.h
MAX_LAUNCH = 65535                # products per call: one launch


def _polys(rng, batch, n, q):
    return [[rng.randrange(q) for _ in range(n)] for _ in range(batch)]


def _max_batch(R, n):
    return min(NOALLOC_SCRATCH_BYTES // (R.k * n * 4), MAX_LAUNCH)


def _noalloc(L, R, A, B, out, batch):
    import torch

    return L.cy_polymul_noalloc(R.h, A.data_ptr(), B.data_ptr(), out.data_ptr(), batch,
                                torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("n,q", [(4096, 2**127 - 1), (1024, 2**61 - 1), (256, 2**127 - 1),
                                 (16384, 2**127 - 1)])
def test_noalloc_matches_polymul_on_consecutive_calls(n, q):
    import torch

    import cuyashe_gb300 as cy

    L = cy.lib()
    R = cy.Ring(n, q)
    batch = min(48, _max_batch(R, n))
    rng = random.Random(n + 1)
    for _ in range(2):  # two calls in a row share (and overwrite) the static scratch
        A, B = R.upload(_polys(rng, batch, n, q)), R.upload(_polys(rng, batch, n, q))
        expected = R.polymul(A, B)
        out = R.empty(batch)
        st = _noalloc(L, R, A, B, out, batch)
        assert st == 0, L.cy_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, expected)


def test_noalloc_matches_the_oracle():
    """Two products checked directly against the schoolbook negacyclic oracle."""
    import torch

    import cuyashe_gb300 as cy

    L = cy.lib()
    n, q = 512, 2**127 - 1
    R = cy.Ring(n, q)
    rng = random.Random(77)
    a, b = _polys(rng, 2, n, q), _polys(rng, 2, n, q)
    out = R.empty(2)
    assert _noalloc(L, R, R.upload(a), R.upload(b), out, 2) == 0, L.cy_last_error()
    torch.cuda.synchronize()
    got = R.download(out)
    for j in range(2):
        assert list(got[j]) == ring.polymul_mod(a[j], b[j], q)


def test_noalloc_rejects_batches_beyond_the_scratch():
    import torch

    import cuyashe_gb300 as cy

    L = cy.lib()
    n, q = 4096, 2**127 - 1
    R = cy.Ring(n, q)
    max_batch = _max_batch(R, n)
    big = max_batch + 1
    A = torch.zeros((big, n, R.L), dtype=torch.int64, device="cuda")
    out = torch.empty_like(A)
    assert _noalloc(L, R, A, A, out, big) == -1
    assert ("at most %d products" % max_batch).encode() in L.cy_last_error()


def test_noalloc_small_rings_capped_at_one_launch():
    """At N = 4 the scratch would hold more than 65535 products; one launch
    cannot, so 65536 are refused with that limit and 65535 run correctly."""
    import numpy as np
    import torch

    import cuyashe_gb300 as cy

    L = cy.lib()
    n, q = 4, 2**61 - 1
    R = cy.Ring(n, q)
    assert NOALLOC_SCRATCH_BYTES // (R.k * n * 4) > MAX_LAUNCH
    A = torch.zeros((MAX_LAUNCH + 1, n, R.L), dtype=torch.int64, device="cuda")
    out = torch.empty_like(A)
    assert _noalloc(L, R, A, A, out, MAX_LAUNCH + 1) == -1
    assert ("at most %d products" % MAX_LAUNCH).encode() in L.cy_last_error()
    rng = np.random.default_rng(4)
    A = torch.from_numpy(rng.integers(0, q, size=(MAX_LAUNCH, n, R.L), dtype=np.int64)).cuda()
    B = torch.from_numpy(rng.integers(0, q, size=(MAX_LAUNCH, n, R.L), dtype=np.int64)).cuda()
    out = torch.empty_like(A)
    assert _noalloc(L, R, A, B, out, MAX_LAUNCH) == 0, L.cy_last_error()
    expected = R.polymul(A, B)
    torch.cuda.synchronize()
    assert torch.equal(out, expected)
