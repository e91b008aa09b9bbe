"""The standalone inverse NTT of length 4096 with its input tile by TMA
(k_intt_tma, schedule ntt=10; its forward is the register schedule's).

Batches from one job to 1500 (more blocks than the GPU holds at once). The
transform must equal the register-exchange schedules bit for bit, invert to
its input, and give the oracle's negacyclic product through the convolution
theorem. Buffers that do not start on 16 bytes are refused. A launch whose
tile wait is made to run out (its barrier told to expect bytes that never
come) reports CY_ERR_TIMEOUT through cy_ntt_check, stores nothing, and leaves
the GPU usable.
"""
import random

import numpy as np
import pytest

from oracle import ring

pytestmark = pytest.mark.gpu

N = 4096
Q127 = ring.largest_prime_below(2**127, 2**16)
TMA = 10  # schedule index of the TMA inverse at N = 4096
TMAS = (TMA,)


@pytest.fixture(scope="module")
def cy():
    import torch

    import cuyashe_gb300

    assert torch.cuda.is_available()
    cuyashe_gb300.lib()
    yield cuyashe_gb300
    cuyashe_gb300.lib().cy_ntt_test_wait(0, 0)
    cuyashe_gb300.tuning_import("n4096.l2.ntt=0")


def _residues(R, jobs, seed):
    import torch

    rng = np.random.default_rng(seed)
    res = np.stack([rng.integers(0, p, size=(jobs, N), dtype=np.int64) for p in R.primes], axis=1)
    return torch.from_numpy(res.astype(np.int32)).cuda()


def _schedule(cy, v):
    cy.tuning_import("n4096.l2.ntt=%d" % v)


@pytest.mark.parametrize("jobs", [1, 7, 1500])
def test_tma_transform_equals_register_schedules(cy, jobs):
    import torch

    R = cy.Ring(N, Q127)
    base = _residues(R, jobs, jobs)
    outs = {}
    for v in (0, 9) + TMAS:
        _schedule(cy, v)
        x = base.clone()
        R.ntt(x)
        outs[v] = x.clone()
        R.ntt(x, inverse=True)
        assert cy.lib().cy_ntt_check() == 0
        assert torch.equal(x, base), "schedule %d does not invert" % v
    _schedule(cy, 0)
    for v in TMAS:
        assert torch.equal(outs[v], outs[0])
        assert torch.equal(outs[v], outs[9])


def test_tma_inverse_equals_register_schedules(cy):
    """The inverse on its own inputs (not a forward output) against schedule 9."""
    import torch

    R = cy.Ring(N, Q127)
    base = _residues(R, 600, 77)
    got = {}
    for v in (9,) + TMAS:
        _schedule(cy, v)
        x = base.clone()
        R.ntt(x, inverse=True)
        got[v] = x
    _schedule(cy, 0)
    for v in TMAS:
        assert torch.equal(got[9], got[v])


@pytest.mark.parametrize("sched", TMAS)
def test_tma_convolution_matches_oracle(cy, sched):
    import torch

    R = cy.Ring(N, Q127)
    rng = random.Random(4)
    jobs = 300
    a = [[rng.randrange(R.q) for _ in range(N)] for _ in range(2)]
    b = [[rng.randrange(R.q) for _ in range(N)] for _ in range(2)]
    # jobs 0 and 1 carry the checked pairs, the rest fills the blocks' job loops
    ra = _residues(R, jobs, 1)
    rb = _residues(R, jobs, 2)
    primes = [int(p) for p in R.primes]
    for j in range(2):
        for i, p in enumerate(primes):
            ra[j, i] = torch.tensor([x % p for x in a[j]], dtype=torch.int64).to(torch.int32)
            rb[j, i] = torch.tensor([x % p for x in b[j]], dtype=torch.int64).to(torch.int32)
    _schedule(cy, sched)
    R.ntt(ra)
    R.ntt(rb)
    pm = torch.tensor(primes, dtype=torch.int64, device="cuda").view(1, -1, 1)
    pr = ((ra.to(torch.int64) * rb.to(torch.int64)) % pm).to(torch.int32)
    R.ntt(pr, inverse=True)
    assert cy.lib().cy_ntt_check() == 0
    _schedule(cy, 0)
    got = pr.cpu().numpy()
    for j in range(2):
        exact = ring.negacyclic_mul_z(a[j], b[j])
        for i, p in enumerate(primes):
            assert [int(v) for v in got[j, i]] == [x % p for x in exact], "job %d prime %d" % (j, i)


def test_unaligned_buffer_refused(cy):
    """Tiles need 16-byte aligned rows; cy_ntt refuses a buffer that does not
    start on 16 bytes (for every schedule) rather than tiling it wrongly."""
    import torch

    R = cy.Ring(N, Q127)
    base = _residues(R, 40, 9)
    flat = torch.zeros(base.numel() + 1, dtype=torch.int32, device="cuda")
    view = flat[1:].view(base.shape)  # 4 bytes past an aligned start
    view.copy_(base)
    _schedule(cy, TMA)
    try:
        with pytest.raises(cy.CyError, match="16-byte aligned"):
            R.ntt(view)
    finally:
        _schedule(cy, 0)
    assert torch.equal(view, base)


@pytest.mark.parametrize("sched", TMAS)
def test_expired_tile_wait_reports_timeout(cy, sched):
    import torch

    lib = cy.lib()
    R = cy.Ring(N, Q127)
    base = _residues(R, 64, 5)
    x = base.clone()
    _schedule(cy, sched)
    assert lib.cy_ntt_check() == 0
    assert lib.cy_ntt_test_wait(2000, 16) == 0
    try:
        R.ntt(x, inverse=True)
        assert lib.cy_ntt_check() == -7  # CY_ERR_TIMEOUT
        assert b"gave up waiting" in lib.cy_last_error()
    finally:
        lib.cy_ntt_test_wait(0, 0)
    assert torch.equal(x, base)  # no block stored anything
    assert lib.cy_ntt_check() == 0  # the record was cleared
    R.ntt(x)
    R.ntt(x, inverse=True)
    assert lib.cy_ntt_check() == 0
    _schedule(cy, 0)
    assert torch.equal(x, base)
