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
Q380 = ring.largest_prime_below(2**380, 2**16)


@pytest.fixture(scope="module")
def setup():
    import torch

    import cuyashe_gb300 as cy
    from cuyashe_gb300.api import Server, Yashe

    assert torch.cuda.is_available()
    ctxs = []
    # the last two are the serving mix's 8192/190-bit and 16384/380-bit classes
    for n, q, t in [(1024, Q62, 257), (2048, Q127, 1024), (4096, Q127, 1024), (1024, Q190, 65537),
                    (8192, Q190, 65537), (16384, Q380, 65537)]:
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
    for i in range(192):
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


def test_device_resident_requests_same_alone_and_in_the_mix(setup):
    """Requests naming ciphertexts already in device memory (uploaded once,
    results left on the device) are gathered, multiplied and scattered on the
    GPU: every result equals the same multiply alone, for every class of the
    serving mix, while host-buffer requests of the same classes run beside them."""
    import torch

    cy, Server, ctxs = setup
    srv = Server(budget_bytes=4 << 30, streams=4, max_batch=32)
    cls = [srv.register(y) for y in ctxs]
    rng = np.random.default_rng(21)
    per = 12
    dev = []
    for k, y in enumerate(ctxs):
        c1 = np.stack([_uniform(rng, y.n, y.q, y.L) for _ in range(per)])
        c2 = np.stack([_uniform(rng, y.n, y.q, y.L) for _ in range(per)])
        d1 = torch.from_numpy(c1.view(np.int64)).cuda()
        d2 = torch.from_numpy(c2.view(np.int64)).cuda()
        do = torch.zeros_like(d1)
        dev.append((k, d1, d2, do))
    torch.cuda.synchronize()
    tickets = []
    host = []
    for k, d1, d2, do in dev:  # device requests of every class, relin on all but the first
        relin = [j > 0 for j in range(per)]
        tickets += srv.submit_device(cls[k], d1, d2, do, relin=relin)
        y = ctxs[k]
        a, b = _uniform(rng, y.n, y.q, y.L), _uniform(rng, y.n, y.q, y.L)
        o = np.zeros_like(a)
        host.append((k, a, b, o, srv.submit(cls[k], a, b, o)))
    for t in tickets:
        srv.wait(t)
    for k, a, b, o, t in host:
        srv.wait(t)
    st = srv.stats()
    assert st.failed == 0 and st.completed == len(tickets) + len(host)
    for k, d1, d2, do in dev:
        y = ctxs[k]
        for j in range(per):
            alone = y.mul(d1[j:j + 1], d2[j:j + 1], relin=j > 0)
            torch.cuda.synchronize()
            assert torch.equal(alone[0], do[j]), "class %d request %d" % (k, j)
    for k, a, b, o, t in host:
        alone = ctxs[k].mul(torch.from_numpy(a.view(np.int64))[None].cuda(),
                            torch.from_numpy(b.view(np.int64))[None].cuda(), relin=True)
        torch.cuda.synchronize()
        assert np.array_equal(alone[0].cpu().numpy().view(np.uint64), o)
    srv.close()


def test_device_requests_refused_on_host(setup):
    import torch

    cy, Server, ctxs = setup
    y = ctxs[0]
    srv = Server(budget_bytes=1 << 30, streams=1, max_batch=4)
    c = srv.register(y)
    d = torch.zeros((2, y.n, y.L), dtype=torch.int64, device="cuda")
    with pytest.raises(cy.CyError):
        srv.submit_device(c + 7, d, d, d)                      # unknown class
    with pytest.raises(cy.CyError):
        srv.submit_device(c, [d.data_ptr() + 8], [d.data_ptr()], [d.data_ptr()])  # not 16-byte aligned
    assert srv.stats().rejected == 2
    srv.close()


def test_wait_deadline_on_a_running_batch(setup):
    """A wait whose deadline passes while its request is still queued or running
    returns CY_ERR_TIMEOUT and leaves the request alone; a later wait succeeds."""
    import torch

    cy, Server, ctxs = setup
    y = ctxs[5]  # N = 16384, 380-bit q: a large batch takes milliseconds on the GPU
    srv = Server(budget_bytes=8 << 30, streams=1, max_batch=128)
    c = srv.register(y)
    rng = np.random.default_rng(5)
    a = np.stack([_uniform(rng, y.n, y.q, y.L) for _ in range(2)])
    d1 = torch.from_numpy(np.repeat(a[:1], 128, axis=0).view(np.int64)).cuda()
    d2 = torch.from_numpy(np.repeat(a[1:], 128, axis=0).view(np.int64)).cuda()
    do = torch.zeros_like(d1)
    torch.cuda.synchronize()
    tickets = srv.submit_device(c, d1, d2, do)
    st = cy.lib().cy_server_wait(srv.h, tickets[-1], 0)  # the deadline has passed at once
    assert st == -7, st
    for t in tickets:
        srv.wait(t, timeout_ms=120000)
    assert srv.stats().completed == 128
    alone = y.mul(d1[:1], d2[:1], relin=True)
    torch.cuda.synchronize()
    assert torch.equal(alone[0], do[127])
    srv.close()
