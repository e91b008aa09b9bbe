"""Serving loop (continuous batching): every result is the same alone and in
the mix; admission respects the device budget; bad requests are refused on the
host.
"""
import threading

import numpy as np
import pytest

from oracle import ring

pytestmark = pytest.mark.gpu

Q62 = ring.largest_prime_below(2**62, 2**16)
Q127 = ring.largest_prime_below(2**127, 2**16)
Q190 = ring.largest_prime_below(2**190, 2**16)


@pytest.fixture(scope="module")
def setup():
    import torch

    import cuyashe_gb300 as cy
    from cuyashe_gb300.api import Server, Yashe

    assert torch.cuda.is_available()
    ctxs = []
    for n, q, t in [(1024, Q62, 257), (2048, Q127, 1024), (4096, Q127, 1024), (1024, Q190, 65537)]:
        y = Yashe(n, q, t)
        y.keygen(n + t)
        ctxs.append(y)
    return cy, Server, ctxs


def _uniform(rng, n, q, L):
    vals = [int(rng.integers(0, 2**62)) * int(rng.integers(1, 2**62)) % q for _ in range(n)]
    from cuyashe_gb300.api import to_limb_array

    return to_limb_array(vals, L)


def test_results_same_alone_and_in_the_mix(setup):
    import torch

    cy, Server, ctxs = setup
    srv = Server(budget_bytes=2 << 30, streams=4, max_batch=32)
    cls = [srv.register(y) for y in ctxs]
    rng = np.random.default_rng(7)
    reqs = []
    for i in range(160):
        c = int(rng.integers(0, len(ctxs)))
        y = ctxs[c]
        c1, c2 = _uniform(rng, y.n, y.q, y.L), _uniform(rng, y.n, y.q, y.L)
        relin = bool(i % 5)
        reqs.append((c, c1, c2, np.zeros_like(c1), relin))
    tickets = [None] * len(reqs)

    def submitter(idx):
        for i in idx:
            c, c1, c2, out, relin = reqs[i]
            tickets[i] = srv.submit(cls[c], c1, c2, out, relin=relin)

    threads = [threading.Thread(target=submitter, args=(range(k, len(reqs), 2),)) for k in range(2)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for t in tickets:
        srv.wait(t)
    st = srv.stats()
    assert st.completed == len(reqs) and st.failed == 0
    assert st.p99_us >= st.p50_us > 0
    for c, c1, c2, out, relin in reqs:
        y = ctxs[c]
        alone = y.mul(torch.from_numpy(c1.view(np.int64))[None].cuda(),
                      torch.from_numpy(c2.view(np.int64))[None].cuda(), relin=relin)
        torch.cuda.synchronize()
        assert np.array_equal(alone[0].cpu().numpy().view(np.uint64), out)
    srv.close()


def test_slot_reused_for_larger_polynomials(setup):
    """One slot serves a batch of many small polynomials, then a batch of a few
    much larger ones: its staging must grow by size in words."""
    import torch

    cy, Server, ctxs = setup
    srv = Server(budget_bytes=2 << 30, streams=1, max_batch=64)
    small, big = ctxs[0], ctxs[2]  # N=1024 / 1 limb, then N=4096 / 2 limbs
    cs, cb = srv.register(small), srv.register(big)
    rng = np.random.default_rng(11)
    items = []
    for _ in range(48):
        c1, c2 = _uniform(rng, small.n, small.q, small.L), _uniform(rng, small.n, small.q, small.L)
        out = np.zeros_like(c1)
        items.append((srv.submit(cs, c1, c2, out), small, c1, c2, out))
    srv.drain()
    for _ in range(10):
        c1, c2 = _uniform(rng, big.n, big.q, big.L), _uniform(rng, big.n, big.q, big.L)
        out = np.zeros_like(c1)
        items.append((srv.submit(cb, c1, c2, out), big, c1, c2, out))
    srv.drain()
    for t, y, c1, c2, out in items:
        srv.wait(t)
        alone = y.mul(torch.from_numpy(c1.view(np.int64))[None].cuda(),
                      torch.from_numpy(c2.view(np.int64))[None].cuda(), relin=True)
        torch.cuda.synchronize()
        assert np.array_equal(alone[0].cpu().numpy().view(np.uint64), out)
    srv.close()


def test_admission_respects_budget(setup):
    cy, Server, ctxs = setup
    y = ctxs[2]  # N = 4096, 127-bit q
    per = 3 * y.n * y.L * 8 + 9 * y.n * 4  # inputs, output and tensor residues of one request
    srv = Server(budget_bytes=3 * per, streams=4, max_batch=64)
    c = srv.register(y)
    rng = np.random.default_rng(3)
    items = []
    for _ in range(40):
        c1, c2 = _uniform(rng, y.n, y.q, y.L), _uniform(rng, y.n, y.q, y.L)
        out = np.zeros_like(c1)
        items.append((srv.submit(c, c1, c2, out), out))
    srv.drain()
    for t, _ in items:
        srv.wait(t)
    st = srv.stats()
    assert st.completed == 40
    assert 0 < st.peak_device_bytes <= 3 * per
    assert st.batches >= 14  # at most three requests in flight at a time
    srv.close()


def test_bad_requests_refused_on_host(setup):
    cy, Server, ctxs = setup
    y = ctxs[0]
    srv = Server(budget_bytes=1 << 20, streams=1, max_batch=4)
    c = srv.register(y)
    a = np.zeros((y.n, y.L), np.uint64)
    assert srv.submit_status(c + 5, a, a, a) == -1           # unknown class
    assert srv.submit_status(c, None, a, a) == -1            # NULL buffer
    tiny = Server(budget_bytes=1024, streams=1, max_batch=4)  # smaller than one request
    c2 = tiny.register(y)
    assert tiny.submit_status(c2, a, a, a) == -4
    assert srv.stats().rejected == 2 and tiny.stats().rejected == 1
    with pytest.raises(cy.CyError):
        srv.wait(123456789)
    srv.close()
    tiny.close()


def test_time_budget_splits_batches(setup):
    """With batch_budget_us a context's batches are capped by its measured time
    per request: a burst is served in more batches, with the same results."""
    import torch

    cy, Server, ctxs = setup
    y = ctxs[2]  # N = 4096, 127-bit q
    rng = np.random.default_rng(11)
    reqs = [(_uniform(rng, y.n, y.q, y.L), _uniform(rng, y.n, y.q, y.L)) for _ in range(8)]
    outs = {}
    for budget in (0, 1):  # 1 us: one request per batch once the estimate exists
        srv = Server(budget_bytes=2 << 30, streams=1, max_batch=256, batch_budget_us=budget)
        c = srv.register(y)
        srv.wait(srv.submit(c, reqs[0][0], reqs[0][1], np.zeros_like(reqs[0][0])))  # first estimate
        srv.reset_stats()
        res = [np.zeros_like(a) for a, _ in reqs * 8]
        tickets = [srv.submit(c, a, b, o) for (a, b), o in zip(reqs * 8, res)]
        for t in tickets:
            srv.wait(t)
        st = srv.stats()
        assert st.completed == len(tickets) and st.failed == 0
        outs[budget] = (res, st.batches)
        srv.close()
    assert outs[1][1] == len(reqs) * 8  # one request per batch under a 1 us budget
    for a, b in zip(outs[0][0], outs[1][0]):
        assert np.array_equal(a, b)
    alone = y.mul(torch.from_numpy(reqs[0][0].view(np.int64))[None].cuda(),
                  torch.from_numpy(reqs[0][1].view(np.int64))[None].cuda(), relin=True)
    torch.cuda.synchronize()
    assert np.array_equal(alone[0].cpu().numpy().view(np.uint64), outs[1][0][0])
    with pytest.raises(cy.CyError):
        Server(budget_bytes=2 << 30, streams=1, max_batch=4, batch_budget_us=-1)
