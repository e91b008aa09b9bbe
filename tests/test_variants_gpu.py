"""Every compiled NTT schedule gives the oracle's product; the autotuner keeps one.

Schedules are forced through ``cy_tuning_import`` ("n<N>.l<limbs>.<op>=<v>")
and each output is compared bit-exactly with the oracle.
"""
import random

import numpy as np

import pytest

from oracle import ring
from oracle.yashe import Yashe as OYashe, YasheParams

pytestmark = pytest.mark.gpu

Q62 = ring.largest_prime_below(2**62, 2**16)
Q127 = ring.largest_prime_below(2**127, 2**16)
Q190 = ring.largest_prime_below(2**190, 2**16)


@pytest.fixture(scope="module")
def cy():
    import torch

    import cuyashe_gb300

    assert torch.cuda.is_available()
    cuyashe_gb300.lib()
    yield cuyashe_gb300
    cuyashe_gb300.tuning_import(";".join("n%d.l%d.%s=0" % (n, l, op) for n in (1024, 2048, 4096, 8192, 16384)
                                         for l in (1, 2, 3, 6) for op in ("mul", "mulc", "ks", "ntt")))


def _variants(cy, n, L, op):
    out = []
    for v in range(32):
        try:
            cy.tuning_import("n%d.l%d.%s=%d" % (n, L, op, v))
        except cy.CyError:
            break
        out.append(v)
    cy.tuning_import("n%d.l%d.%s=0" % (n, L, op))
    return out


@pytest.mark.parametrize("n,q", [(1024, Q62), (2048, Q127), (4096, Q127), (4096, Q190), (8192, Q127),
                                 (16384, Q62)])
def test_every_product_schedule_matches_oracle(cy, n, q):
    import torch

    R = cy.Ring(n, q)
    rng = random.Random(n)
    # three jobs: schedules with two jobs per block also meet an odd tail
    a = [[rng.randrange(q) for _ in range(n)] for _ in range(3)]
    b = [[rng.randrange(q) for _ in range(n)] for _ in range(3)]
    A, B = R.upload(a), R.upload(b)
    exp = [ring.polymul_mod(a[j], b[j], q) for j in range(3)]
    vs = _variants(cy, n, R.L, "mul")
    assert vs and vs[0] == 0
    for v in vs:
        cy.tuning_import("n%d.l%d.mul=%d" % (n, R.L, v))
        out = R.download(R.polymul(A, B))
        torch.cuda.synchronize()
        for j in range(3):
            assert list(out[j]) == exp[j], "schedule %d" % v
    cy.tuning_import("n%d.l%d.mul=0" % (n, R.L))


def test_every_tensor_and_keyswitch_schedule_matches_oracle(cy):
    import torch

    n, q, t = 4096, Q127, 1024
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    keys = oy.keygen(5)
    rng = random.Random(6)
    c1 = [rng.randrange(q) for _ in range(n)]
    c2 = [rng.randrange(q) for _ in range(n)]
    exp_t = oy.mul_tensor(c1, c2)
    exp_r = oy.keyswitch(keys, exp_t)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    C1, C2 = R.upload([c1]), R.upload([c2])
    for v in _variants(cy, n, R.L, "mulc"):
        cy.tuning_import("n%d.l%d.mulc=%d" % (n, R.L, v))
        out = R.download(Y.mul(C1, C2, relin=False))
        torch.cuda.synchronize()
        assert list(out[0]) == exp_t, "tensor schedule %d" % v
    for v in _variants(cy, n, R.L, "ks"):
        cy.tuning_import("n%d.l%d.ks=%d" % (n, R.L, v))
        out = R.download(Y.keyswitch(R.upload([exp_t])))
        torch.cuda.synchronize()
        assert list(out[0]) == exp_r, "keyswitch schedule %d" % v
        # inside the HE multiply the keyswitch reads the tensor product limb-major
        out = R.download(Y.mul(C1, C2, relin=True))
        torch.cuda.synchronize()
        assert list(out[0]) == exp_r, "keyswitch schedule %d inside the HE multiply" % v
    cy.tuning_import("n%d.l%d.mulc=0;n%d.l%d.ks=0" % (n, R.L, n, R.L))


def test_every_keyswitch_schedule_at_16384_matches_oracle(cy):
    """N = 16384, 380-bit q (12 digits, six-limb kernels): the four-digit pass does
    not fit in shared memory, so each schedule runs its small-digit kernel (two
    digits per pass, or one). The keyswitch is a fixed function of c and the
    evaluation keys, so random keys stand in for generated ones."""
    import torch

    from oracle.yashe import YasheKeys

    n, t = 16384, 1024
    q = ring.largest_prime_below(2**380, 2**16)
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    rng = random.Random(16)
    ell = oy.p.ell
    evk = [[rng.randrange(q) for _ in range(n)] for _ in range(ell)]
    keys = YasheKeys(f=[1] + [0] * (n - 1), h=[0] * n, evk=evk)
    c = [rng.randrange(q) for _ in range(n)]
    exp = oy.keyswitch(keys, c)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    assert Y.ell == ell == 12 and R.L == 6
    C = R.upload([c])
    vs = _variants(cy, n, R.L, "ks")
    assert len(vs) >= 2
    for v in vs:
        cy.tuning_import("n%d.l%d.ks=%d" % (n, R.L, v))
        out = R.download(Y.keyswitch(C))
        torch.cuda.synchronize()
        assert list(out[0]) == exp, "keyswitch schedule %d" % v
    cy.tuning_import("n%d.l%d.ks=0" % (n, R.L))


def test_autotune_chooses_and_exports(cy):
    import torch

    n, q, t = 4096, Q127, 1024
    Y = cy.Yashe(n, q, t)
    Y.autotune(batch=64)
    spec = cy.tuning_export()
    for op in ("mul", "mulc", "ks"):
        assert ("n4096.l2.%s=" % op) in spec
    cy.tuning_import(spec)
    assert cy.tuning_export() == spec
    with pytest.raises(cy.CyError):
        cy.tuning_import("n4096.l2.mul=99")
    with pytest.raises(cy.CyError):
        cy.tuning_import("garbage")
    torch.cuda.synchronize()


@pytest.mark.parametrize("n,q", [(1024, Q62), (4096, Q127), (8192, Q127), (16384, Q62)])
def test_every_ntt_schedule_agrees(cy, n, q):
    """cy_ntt under every schedule: the same forward transform as the default,
    and the inverse gives the input back (5 jobs: two per block plus one alone)."""
    import torch

    R = cy.Ring(n, q)
    rng = np.random.default_rng(n)
    res = np.stack([rng.integers(0, p, size=(5, n), dtype=np.int64) for p in R.primes], axis=1).astype(np.int32)
    base = torch.from_numpy(res).cuda()
    vs = _variants(cy, n, R.L, "ntt")
    outs = []
    for v in vs:
        cy.tuning_import("n%d.l%d.ntt=%d" % (n, R.L, v))
        x = base.clone()
        R.ntt(x)
        outs.append(x.clone())
        R.ntt(x, inverse=True)
        assert torch.equal(x, base)
    cy.tuning_import("n%d.l%d.ntt=0" % (n, R.L))
    assert all(torch.equal(o, outs[0]) for o in outs)
