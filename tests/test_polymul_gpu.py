"""GPU parity: multiplication in Z_q[x]/(x^N+1) through the C ABI vs the oracle.

Bit-exact: every coefficient of every product equals the oracle's
``[fold(a*b)]_q`` (exact integers). Sizes where the Python oracle is slow are
covered by size-independent properties (commutativity, distributivity,
multiplication by x^k as a negacyclic shift).
"""
import json
import os
import random

import numpy as np
import pytest

from oracle import ring

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))

Q127 = 2**127 - 1                              # benchmark_polynomial.cpp:109-110
Q62 = ring.largest_prime_below(2**62)
Q190 = ring.largest_prime_below(2**190)
Q380 = ring.largest_prime_below(2**380)
QREF96 = int(GOLD["poly_suite"]["q"])          # test.cu PolySuite modulus


@pytest.fixture(scope="module")
def cy():
    import torch

    import cuyashe_gb300

    assert torch.cuda.is_available()
    cuyashe_gb300.lib()
    return cuyashe_gb300


def _rand_polys(rng, batch, n, q):
    return [[rng.randrange(q) for _ in range(n)] for _ in range(batch)]


def _gpu_mul(cy, n, q, a, b):
    import torch

    R = cy.Ring(n, q)
    out = R.download(R.polymul(R.upload(a), R.upload(b)))
    torch.cuda.synchronize()
    return R, out


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
@pytest.mark.parametrize("q", [Q127, Q62, QREF96])
def test_polymul_matches_oracle(cy, n, q):
    rng = random.Random(n * 7919 + q % 1000)
    batch = 3 if n <= 1024 else 2
    a, b = _rand_polys(rng, batch, n, q), _rand_polys(rng, batch, n, q)
    R, out = _gpu_mul(cy, n, q, a, b)
    assert R.k >= 2
    for j in range(batch):
        assert list(out[j]) == ring.polymul_mod(a[j], b[j], q)


@pytest.mark.parametrize("n,q", [(8192, Q127), (1024, Q190), (2048, Q380), (64, 97), (16, 2**31 - 1),
                                 (256, 2**64 - 59), (8, 3)])
def test_polymul_other_moduli(cy, n, q):
    rng = random.Random(n + 17)
    a, b = _rand_polys(rng, 2, n, q), _rand_polys(rng, 2, n, q)
    _, out = _gpu_mul(cy, n, q, a, b)
    for j in range(2):
        assert list(out[j]) == ring.polymul_mod(a[j], b[j], q)


def test_golden_test_mul_2_plain_product(cy):
    """src/test_mul.cu second test. With N = 16 > deg(a*b) and q > every product
    coefficient the negacyclic product mod q is the plain product over Z."""
    t = GOLD["test_mul_2"]
    a = [int(x) for x in t["a"]]
    b = [int(x) for x in t["b"]]
    exp = [int(x) for x in t["expected_plain_product"]]
    q = ring.largest_prime_below(2**140)
    n = 16
    _, out = _gpu_mul(cy, n, q, [a + [0] * (n - len(a))], [b + [0] * (n - len(b))])
    assert list(out[0][: len(exp)]) == exp
    assert all(v == 0 for v in out[0][len(exp):])


def test_golden_simple_multiply(cy):
    """src/test.cu:421-470: a_i = i, b_i = 1 at degree 8, q = PolySuite modulus."""
    n, q = 16, QREF96
    a = list(range(8)) + [0] * 8
    b = [1] * 8 + [0] * 8
    _, out = _gpu_mul(cy, n, q, [a], [b])
    assert list(out[0][:15]) == ring.plain_mul(list(range(8)), [1] * 8)


def test_polysuite_random_n8(cy):
    """PolySuite-style randomized products at N = 8 (src/test.cu:472-628)."""
    ps = GOLD["poly_suite"]
    q, n = int(ps["q"]), ps["degree"]
    rng = random.Random(ps["srand"])
    a, b = _rand_polys(rng, ps["ntests"], n, q), _rand_polys(rng, ps["ntests"], n, q)
    _, out = _gpu_mul(cy, n, q, a, b)
    for j in range(ps["ntests"]):
        assert list(out[j]) == ring.polymul_mod(a[j], b[j], q)


def test_edge_values(cy):
    n, q = 1024, Q127
    zeros = [[0] * n]
    maxv = [[q - 1] * n]
    one = [[1] + [0] * (n - 1)]
    rng = random.Random(5)
    r = _rand_polys(rng, 1, n, q)
    _, out = _gpu_mul(cy, n, q, zeros + maxv + one + maxv, r + maxv + r + one)
    assert list(out[0]) == [0] * n
    assert list(out[1]) == ring.polymul_mod(maxv[0], maxv[0], q)
    assert list(out[2]) == r[0]
    assert list(out[3]) == maxv[0]


def test_batch_zero_and_large_batch(cy):
    import torch

    n, q = 256, Q127
    R = cy.Ring(n, q)
    e = R.empty(0)
    R.polymul(e, e, out=R.empty(0))
    rng = random.Random(11)
    batch = 700  # more than one chunk is not needed here; exercises the grid.y range
    a, b = _rand_polys(rng, batch, n, q), _rand_polys(rng, batch, n, q)
    out = R.download(R.polymul(R.upload(a), R.upload(b)))
    torch.cuda.synchronize()
    for j in [0, 1, 349, 698, 699]:
        assert list(out[j]) == ring.polymul_mod(a[j], b[j], q)


def test_invalid_arguments(cy):
    import ctypes

    R = cy.Ring(64, Q127)
    L = cy.lib()
    assert L.cy_polymul(R.h, None, None, None, 1, None) == -1
    assert L.cy_polymul(R.h, None, None, None, -1, None) == -1
    assert L.cy_polymul(R.h, None, None, None, 0, None) == 0
    h = ctypes.c_void_p()
    assert L.cy_ring_create(100, cy.limbs_of(Q127, 2), 2, ctypes.byref(h)) == -2


def test_full_size_properties_n16384_q380(cy):
    """Size-independent properties at the deep-level ring (N = 16384, 380-bit q):
    commutativity, distributivity, and x^k * a = negacyclic shift of a; plus one
    exact comparison with the Kronecker oracle."""
    import torch

    n, q = 16384, Q380
    R = cy.Ring(n, q)
    rng = random.Random(3)
    a, b, c = (_rand_polys(rng, 1, n, q) for _ in range(3))
    A, B, C = R.upload(a), R.upload(b), R.upload(c)
    ab = R.polymul(A, B)
    ba = R.polymul(B, A)
    lhs = R.polymul(A, R.polyadd(B, C))
    rhs = R.polyadd(ab, R.polymul(A, C))
    k = 12345
    xk = [[0] * n]
    xk[0][k] = 1
    shifted = R.download(R.polymul(A, R.upload(xk)))
    torch.cuda.synchronize()
    assert torch.equal(ab, ba)
    assert torch.equal(lhs, rhs)
    exp_shift = [(-a[0][i - k + n]) % q if i < k else a[0][i - k] for i in range(n)]
    assert list(shifted[0]) == exp_shift
    assert list(R.download(ab)[0]) == ring.polymul_mod(a[0], b[0], q)


def test_add_sub_scalar(cy):
    import torch

    rng = random.Random(21)
    for n, q in [(64, Q127), (128, Q190), (32, Q62), (16, Q380)]:
        R = cy.Ring(n, q)
        a, b = _rand_polys(rng, 3, n, q), _rand_polys(rng, 3, n, q)
        a[0][0], b[0][0] = q - 1, q - 1
        A, B = R.upload(a), R.upload(b)
        s = rng.randrange(q)
        add, sub, sc = R.download(R.polyadd(A, B)), R.download(R.polysub(A, B)), R.download(R.scalar_mul(A, s))
        torch.cuda.synchronize()
        for j in range(3):
            assert list(add[j]) == [(x + y) % q for x, y in zip(a[j], b[j])]
            assert list(sub[j]) == [(x - y) % q for x, y in zip(a[j], b[j])]
            assert list(sc[j]) == [(x * s) % q for x in a[j]]


def test_crt_ntt_icrt_roundtrip(cy):
    """CRT split, forward NTT, inverse NTT and ICRT give back the input, and the
    inverse NTT of a pointwise product of forward NTTs is the negacyclic product."""
    import torch

    n, q = 4096, Q127
    R = cy.Ring(n, q)
    rng = random.Random(4)
    a = _rand_polys(rng, 2, n, q)
    A = R.upload(a)
    res = R.crt(A)
    primes = R.primes
    r_host = res.cpu().numpy().view(np.uint32)
    for i, p in enumerate(primes):
        assert [int(v) for v in r_host[0, i, :8]] == [x % p for x in a[0][:8]]
    R.ntt(res)
    R.ntt(res, inverse=True)
    back = R.download(R.icrt(res))
    torch.cuda.synchronize()
    assert [list(x) for x in back] == a
    # INTT(NTT(a) . NTT(b)) is the exact negacyclic product reduced mod each prime
    b = _rand_polys(rng, 2, n, q)
    ra, rb = R.crt(A), R.crt(R.upload(b))
    R.ntt(ra)
    R.ntt(rb)
    prod = ra.cpu().numpy().view(np.uint32).astype(np.uint64) * rb.cpu().numpy().view(np.uint32).astype(np.uint64)
    for i, p in enumerate(primes):
        prod[:, i, :] %= p
    pr = torch.from_numpy(prod.astype(np.uint32).view(np.int32)).cuda()
    R.ntt(pr, inverse=True)
    exact = [ring.negacyclic_mul_z(a[j], b[j]) for j in range(2)]
    got = pr.cpu().numpy().view(np.uint32)
    for j in range(2):
        for i, p in enumerate(primes):
            assert [int(v) for v in got[j, i, :16]] == [x % p for x in exact[j][:16]]


def test_polymul_host_entry_point(cy):
    n, q = 512, Q127
    R = cy.Ring(n, q)
    rng = random.Random(8)
    a, b = _rand_polys(rng, 2, n, q), _rand_polys(rng, 2, n, q)
    from cuyashe_gb300.api import from_limb_array, to_limb_array

    out = from_limb_array(R.polymul_host(to_limb_array(a, 2), to_limb_array(b, 2)))
    for j in range(2):
        assert list(out[j]) == ring.polymul_mod(a[j], b[j], q)


def test_batched_mixed_rings_same_as_alone(cy):
    """Config-3 style mixed submission: every product equals the product alone."""
    import torch

    rng = random.Random(33)
    specs = [(1024, Q62), (2048, Q127), (4096, Q190), (8192, Q62), (1024, Q127)]
    rings = [cy.Ring(n, q) for n, q in specs]
    jobs, refs, whole = [], [], []
    for R, (n, q) in zip(rings, specs):
        a, b = _rand_polys(rng, 3, n, q), _rand_polys(rng, 3, n, q)
        A, B = R.upload(a), R.upload(b)
        C = R.empty(3)
        for j in range(3):  # one job per product; contiguous jobs of a ring share a launch
            jobs.append((R, A[j:j + 1], B[j:j + 1], C[j:j + 1]))
        whole.append((R, A, B, C))
        refs.append((a, b, q))
    jobs = jobs[::2] + jobs[1::2]  # interleave rings so that grouping is exercised
    from cuyashe_gb300.api import polymul_batched

    polymul_batched(jobs)
    torch.cuda.synchronize()
    for (R, A, B, C), (a, b, q) in zip(whole, refs):
        alone = R.polymul(A, B)
        torch.cuda.synchronize()
        assert torch.equal(alone, C)
        got = R.download(C)
        for j in range(3):
            assert list(got[j]) == ring.polymul_mod(a[j], b[j], q)


def test_mixed_batch_one_launch_config3(cy):
    """512 products, N uniform over {1024, 2048, 4096, 8192}, q of 62/127/190 bits:
    one persistent launch; every product equals the per-ring result, a sample
    equals the oracle; rings outside the mixed kernel's range (N = 16384, a
    380-bit q) ride along in the same submission."""
    import torch

    from cuyashe_gb300.api import polymul_batched, polymul_batched_status

    rng = random.Random(512)
    qs = [Q62, Q127, Q190]
    ns = [1024, 2048, 4096, 8192]
    rings = {(n, q): cy.Ring(n, q) for n in ns for q in qs}
    rings[(16384, Q62)] = cy.Ring(16384, Q62)
    rings[(1024, Q380)] = cy.Ring(1024, Q380)
    specs = [(rng.choice(ns), rng.choice(qs)) for _ in range(512)] + [(16384, Q62), (1024, Q380)]
    jobs, data = [], []
    for n, q in specs:
        R = rings[(n, q)]
        a = [rng.randrange(q) for _ in range(n)]
        b = [rng.randrange(q) for _ in range(n)]
        A, B = R.upload([a]), R.upload([b])
        C = R.empty(1)
        jobs.append((R, A, B, C))
        data.append((a, b, q))
    polymul_batched(jobs)
    polymul_batched_status()
    torch.cuda.synchronize()
    for (R, A, B, C) in jobs:
        assert torch.equal(R.polymul(A, B), C)
    for idx in [0, 1, 7, 100, 255, 511, 512, 513]:
        R, A, B, C = jobs[idx]
        a, b, q = data[idx]
        assert list(R.download(C)[0]) == ring.polymul_mod(a, b, q)
    # a second submission on the same scratch
    polymul_batched(jobs[:64])
    polymul_batched_status()
    for (R, A, B, C) in jobs[:64]:
        assert torch.equal(R.polymul(A, B), C)


def test_prepared_mixed_batch_reruns_on_new_inputs(cy):
    """A MixedBatch built once gives the per-ring products on every run, also
    after its input buffers are refilled in place."""
    import torch

    from cuyashe_gb300.api import MixedBatch, polymul_batched_status

    rng = np.random.default_rng(77)
    specs = [(1024, Q62), (2048, Q127), (4096, Q190), (8192, Q127), (4096, Q127)] * 8
    rings = {s: cy.Ring(*s) for s in set(specs)}

    def fill(R, t):
        L = R.L
        top = R.q.bit_length() - 64 * (L - 1) - 1
        x = rng.integers(0, 2**63, size=(1, R.n, L), dtype=np.uint64)
        x[..., L - 1] &= np.uint64((1 << top) - 1)
        t.copy_(torch.from_numpy(x.view(np.int64)).cuda())

    jobs = []
    for s in specs:
        R = rings[s]
        A, B, C = R.empty(1), R.empty(1), R.empty(1)
        fill(R, A)
        fill(R, B)
        jobs.append((R, A, B, C))
    mb = MixedBatch(jobs)
    assert len(mb) == len(jobs)
    for _ in range(2):
        mb.run()
        polymul_batched_status()
        for (R, A, B, C) in jobs:
            assert torch.equal(R.polymul(A, B), C)
        for (R, A, B, C) in jobs:  # new inputs, same buffers
            fill(R, A)
