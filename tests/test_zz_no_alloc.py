"""The allocation-free product (cy_polymul_noalloc) against cy_polymul.

cy_polymul_noalloc exists for callers that may not call cudaMalloc -- code
recorded into a CUDA graph, serving paths that cannot take cudaMalloc's
device-wide synchronisation, hosts whose device memory belongs to another
allocator. It keeps its scratch in a fixed array inside the library instead of
a workspace. Its results must equal the ordinary entry point's bit for bit, on
consecutive calls that reuse the shared array, and batches too large for the
array must be refused with a clear message.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes when run alone.
"""
import random

import pytest

pytestmark = pytest.mark.gpu

NOALLOC_SCRATCH_BYTES = 16 << 20  # CY_NOALLOC_SCRATCH_BYTES in include/cuyashe.h


def _polys(rng, batch, n, q):
    return [[rng.randrange(q) for _ in range(n)] for _ in range(batch)]


@pytest.mark.parametrize("n,q", [(4096, 2**127 - 1), (1024, 2**61 - 1)])
def test_noalloc_matches_polymul_on_consecutive_calls(n, q):
    import torch

    import cuyashe_gb300 as cy

    L = cy.lib()
    R = cy.Ring(n, q)
    max_batch = NOALLOC_SCRATCH_BYTES // (R.k * n * 4)
    batch = min(48, max_batch)
    rng = random.Random(n + 1)
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # two calls in a row share (and overwrite) the static scratch
        A, B = R.upload(_polys(rng, batch, n, q)), R.upload(_polys(rng, batch, n, q))
        expected = R.polymul(A, B)
        out = R.empty(batch)
        st = L.cy_polymul_noalloc(R.h, A.data_ptr(), B.data_ptr(), out.data_ptr(), batch, stream)
        assert st == 0, L.cy_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, expected)


def test_noalloc_rejects_batches_beyond_the_scratch():
    import torch

    import cuyashe_gb300 as cy

    L = cy.lib()
    n, q = 4096, 2**127 - 1
    R = cy.Ring(n, q)
    max_batch = NOALLOC_SCRATCH_BYTES // (R.k * n * 4)
    big = max_batch + 1
    A = torch.zeros((big, n, R.L), dtype=torch.int64, device="cuda")
    out = torch.empty_like(A)
    st = L.cy_polymul_noalloc(R.h, A.data_ptr(), A.data_ptr(), out.data_ptr(), big,
                              torch.cuda.current_stream().cuda_stream)
    assert st == -1
    assert ("at most %d products" % max_batch).encode() in L.cy_last_error()
