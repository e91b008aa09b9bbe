"""CUDA graphs of a fixed batch replay the same results as direct calls, also
after the input buffers are refilled."""
import numpy as np
import pytest

from oracle import ring

pytestmark = pytest.mark.gpu

Q127 = ring.largest_prime_below(2**127, 2**16)


def _rand(R, batch, seed):
    rng = np.random.default_rng(seed)
    lo = rng.integers(0, 2**64, size=(batch, R.n), dtype=np.uint64)
    hi = rng.integers(0, 2**62, size=(batch, R.n), dtype=np.uint64)
    return R.upload(np.stack([lo, hi], axis=-1))


def test_polymul_and_yashe_graphs():
    import torch

    import cuyashe_gb300 as cy

    R = cy.Ring(4096, 2**127 - 1)
    A, B = _rand(R, 300, 1), _rand(R, 300, 2)
    out = R.empty(300)
    g = R.polymul_graph(A, B, out)
    for seed in (3, 4):
        g.launch()
        torch.cuda.synchronize()
        assert torch.equal(out, R.polymul(A, B))
        A.copy_(_rand(R, 300, seed))  # same buffers, new contents

    Y = cy.Yashe(4096, Q127, 1024)
    Y.keygen(11)
    C1, C2 = _rand(Y.ring, 64, 5), _rand(Y.ring, 64, 6)
    o = Y.ring.empty(64)
    gy = Y.mul_graph(C1, C2, o, relin=True)
    for seed in (7, 8):
        gy.launch()
        torch.cuda.synchronize()
        assert torch.equal(o, Y.mul(C1, C2, relin=True))
        C2.copy_(_rand(Y.ring, 64, seed))


def test_multi_chunk_yashe_graph_matches_direct_calls():
    """500 pairs are several chunks, captured on two streams (fork/join events)."""
    import torch

    import cuyashe_gb300 as cy

    Y = cy.Yashe(4096, Q127, 1024)
    Y.keygen(12)
    C1, C2 = _rand(Y.ring, 500, 9), _rand(Y.ring, 500, 10)
    o = Y.ring.empty(500)
    g = Y.mul_graph(C1, C2, o, relin=True)
    s = torch.cuda.Stream()
    for seed in (13, 14):
        s.wait_stream(torch.cuda.current_stream())  # inputs written on the current stream
        g.launch(s)
        s.synchronize()
        assert torch.equal(o, Y.mul(C1, C2, relin=True))
        C1.copy_(_rand(Y.ring, 500, seed))
