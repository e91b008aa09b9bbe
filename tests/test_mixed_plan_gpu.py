"""Prepared mixed batches (cy_mixed_plan_*): polynomial products and YASHE
multiplies of different N and CRT depth in one persistent launch.

Every job's result must equal the same operation alone (cy_polymul /
cy_yashe_mul, themselves checked against the oracle elsewhere) bit for bit,
under both schedules of the mixed kernel, on graph replays with new inputs,
and the HE products must decrypt to m1*m2 mod t. A plan whose bounded wait is
made to expire reports CY_ERR_TIMEOUT and leaves the GPU usable.
"""
import random

import numpy as np
import pytest

from oracle import ring

pytestmark = pytest.mark.gpu

Q62 = ring.largest_prime_below(2**62, 2**16)
Q127 = ring.largest_prime_below(2**127, 2**16)
Q190 = ring.largest_prime_below(2**190, 2**16)

# (N, q, t) of the YASHE classes: t = 17 for the 62-bit q (noise budget)
HE_CLASSES = [(2048, Q62, 17), (4096, Q127, 1024), (8192, Q190, 65537), (1024, Q190, 65537)]
PRODUCT_CLASSES = [(1024, Q62), (2048, Q127), (4096, Q190), (8192, Q127), (4096, 2**127 - 1)]


@pytest.fixture(scope="module")
def ctx():
    import torch

    import cuyashe_gb300 as cy
    from cuyashe_gb300.api import Yashe

    assert torch.cuda.is_available()
    cy.lib()
    schemes = []
    for n, q, t in HE_CLASSES:
        y = Yashe(n, q, t)
        y.keygen(n + t)
        schemes.append(y)
    rings = [cy.Ring(n, q) for n, q in PRODUCT_CLASSES]
    return cy, schemes, rings


def _random(R, batch, rng):
    import torch

    return R.upload([[rng.randrange(R.q) for _ in range(R.n)] for _ in range(batch)])


def _build(ctx, seed, per=3):
    """Jobs of every class, interleaved: products on uniform inputs, HE multiplies
    (relinearised and not) on fresh GPU encryptions of uniform plaintexts."""
    import torch

    cy, schemes, rings = ctx
    rng = random.Random(seed)
    jobs, expect = [], []
    for i in range(per):
        for R in rings:
            a, b = _random(R, 1, rng), _random(R, 1, rng)
            c = R.empty(1)
            jobs.append(("mul", R, a, b, c))
            expect.append(("mul", R, a, b, c))
        for y in schemes:
            m1 = torch.from_numpy(np.array([[rng.randrange(y.t) for _ in range(y.n)]], np.int64)).cuda()
            m2 = torch.from_numpy(np.array([[rng.randrange(y.t) for _ in range(y.n)]], np.int64)).cuda()
            c1, c2 = y.encrypt(m1, seed=rng.randrange(1 << 30)), y.encrypt(m2, seed=rng.randrange(1 << 30))
            out = y.ring.empty(1)
            relin = i != 1
            jobs.append(("yashe", y, c1, c2, out, relin))
            expect.append(("yashe", y, c1, c2, out, relin, m1, m2))
    return jobs, expect


def _check(ctx, expect, decrypt=True):
    import torch

    cy, schemes, rings = ctx
    for e in expect:
        if e[0] == "mul":
            _, R, a, b, c = e
            alone = R.polymul(a, b)
            torch.cuda.synchronize()
            assert torch.equal(alone, c), "product N=%d" % R.n
        else:
            _, y, c1, c2, out, relin, m1, m2 = e
            alone = y.mul(c1, c2, relin=relin)
            torch.cuda.synchronize()
            assert torch.equal(alone, out), "HE multiply N=%d relin=%d" % (y.n, relin)
            if decrypt:
                got = y.decrypt(out, aftermul=not relin).cpu().numpy().view(np.uint64)[0]
                exp = ring.polymul_mod([int(v) for v in m1[0].cpu()], [int(v) for v in m2[0].cpu()], y.t)
                assert [int(v) for v in got] == exp, "decryption N=%d relin=%d" % (y.n, relin)


def test_products_and_he_multiplies_in_one_launch_match_alone(ctx):
    cy = ctx[0]
    jobs, expect = _build(ctx, 11)
    plan = cy.MixedPlan(jobs)
    for sched in (0, 1):
        for e in expect:  # clear the outputs so that each schedule writes them afresh
            e[4].zero_()
        plan.schedule = sched
        before = cy.launch_count()
        plan.launch()
        assert cy.launch_count() - before == 1  # one kernel for the whole batch
        plan.status()
        _check(ctx, expect, decrypt=sched == 0)


def test_product_matches_the_oracle(ctx):
    import torch

    cy, schemes, rings = ctx
    R = rings[0]  # N = 1024, 62-bit q
    rng = random.Random(3)
    a = [[rng.randrange(R.q) for _ in range(R.n)]]
    b = [[rng.randrange(R.q) for _ in range(R.n)]]
    c = R.empty(1)
    plan = cy.MixedPlan([("mul", R, R.upload(a), R.upload(b), c)])
    plan.launch()
    plan.status()
    assert list(R.download(c)[0]) == ring.polymul_mod(a[0], b[0], R.q)


def test_graph_replay_with_new_inputs(ctx):
    """The launch allocates nothing and waits for nothing on the host, so it is
    recorded once and replayed; inputs rewritten in place between replays."""
    import torch

    cy = ctx[0]
    jobs, expect = _build(ctx, 12, per=1)
    plan = cy.MixedPlan(jobs)
    plan.launch()
    plan.status()
    g = plan.graph()
    rng = random.Random(99)
    mem0 = torch.cuda.memory_allocated()
    for rep in range(2):
        for e in expect:
            if e[0] == "mul":
                R = e[1]
                e[2].copy_(_random(R, 1, rng))
                e[3].copy_(_random(R, 1, rng))
            e[4].zero_()
        torch.cuda.synchronize()
        g.launch()
        plan.status()
        _check(ctx, expect, decrypt=False)
    assert torch.cuda.memory_allocated() == mem0


def test_autotune_keeps_a_schedule_with_identical_results(ctx):
    cy = ctx[0]
    jobs, expect = _build(ctx, 13, per=2)
    plan = cy.MixedPlan(jobs)
    s = plan.autotune()
    assert s in (0, 1) and plan.schedule == s
    for e in expect:
        e[4].zero_()
    plan.launch()
    plan.status()
    _check(ctx, expect, decrypt=False)


def test_bad_plans_refused(ctx):
    cy, schemes, rings = ctx
    R = rings[0]
    a = R.empty(1)
    with pytest.raises(cy.CyError):
        cy.MixedPlan([("mul", R, a, a, a)])  # output aliases an input
    big = cy.Ring(16384, Q62)
    b = big.empty(1)
    with pytest.raises(cy.CyError):
        cy.MixedPlan([("mul", big, b, big.empty(1), big.empty(1))])  # N outside 1024..8192
    plan = cy.MixedPlan([("mul", R, R.empty(1), R.empty(1), R.empty(1))])
    with pytest.raises(cy.CyError):
        plan.schedule = 2


def test_expired_wait_reports_timeout(ctx):
    """A job made to wait for one transform more than it has: its epilogue gives
    up after a short bounded spin, the launch ends, the status says timeout, the
    other jobs of the plan are intact, and the GPU keeps working."""
    import torch

    cy, schemes, rings = ctx
    rng = random.Random(5)
    R0, R1 = rings[1], rings[2]
    a0, b0, c0 = _random(R0, 1, rng), _random(R0, 1, rng), R0.empty(1)
    a1, b1, c1 = _random(R1, 1, rng), _random(R1, 1, rng), R1.empty(1)
    plan = cy.MixedPlan([("mul", R0, a0, b0, c0), ("mul", R1, a1, b1, c1)])
    assert cy.lib().cy_mixed_plan_test_starve(plan.h, 0, 2000) == 0
    plan.launch()
    assert plan.status_code() == -7  # CY_ERR_TIMEOUT
    assert b"gave up waiting" in cy.lib().cy_last_error()
    alone = R1.polymul(a1, b1)
    torch.cuda.synchronize()
    assert torch.equal(alone, c1)
