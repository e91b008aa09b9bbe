"""GPU parity of the YASHE homomorphic multiply, keyswitch and decryption.

Keys and ciphertexts come from the oracle (BLLN13 restatement, oracle/yashe.py);
every GPU output is compared bit-exactly with the oracle's. The product's own
host keygen/encryption is checked by decrypting through the oracle.
"""
import json
import os
import random

import numpy as np
import pytest

from oracle import ring
from oracle.yashe import Sampler, Yashe as OYashe, YasheParams

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))
Q127 = ring.largest_prime_below(2**127, 2**16)
Q62 = ring.largest_prime_below(2**62, 2**16)
Q190 = ring.largest_prime_below(2**190, 2**16)
Q380 = ring.largest_prime_below(2**380, 2**16)


@pytest.fixture(scope="module")
def cy():
    import torch

    import cuyashe_gb300

    assert torch.cuda.is_available()
    cuyashe_gb300.lib()
    return cuyashe_gb300


_CACHE = {}


def _setup(n, q, t, seed=1):
    key = (n, q, t, seed)
    if key not in _CACHE:
        oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
        keys = oy.keygen(seed)
        smp = Sampler(seed + 100)
        pts = [smp.uniform(n, t) for _ in range(4)]
        cts = [oy.encrypt(keys, m, seed + 200 + i) for i, m in enumerate(pts)]
        _CACHE[key] = (oy, keys, pts, cts)
    return _CACHE[key]


@pytest.mark.parametrize("n,q,t", [(16, Q127, 1024), (1024, Q127, 1024), (4096, Q127, 1024), (256, Q62, 257),
                                   (512, Q190, 65537)])
def test_yashe_mul_matches_oracle(cy, n, q, t):
    import torch

    oy, keys, pts, cts = _setup(n, q, t)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    C1, C2 = R.upload([cts[0], cts[2]]), R.upload([cts[1], cts[3]])
    tensor = R.download(Y.mul(C1, C2, relin=False))
    relin = R.download(Y.mul(C1, C2, relin=True))
    ks = R.download(Y.keyswitch(R.upload([list(tensor[0])])))
    torch.cuda.synchronize()
    for j, (a, b) in enumerate([(0, 1), (2, 3)]):
        exp_tensor = oy.mul_tensor(cts[a], cts[b])
        assert list(tensor[j]) == exp_tensor
        exp_relin = oy.keyswitch(keys, exp_tensor)
        assert list(relin[j]) == exp_relin
        assert oy.decrypt(keys, exp_relin) == ring.polymul_mod(pts[a], pts[b], t)
    assert list(ks[0]) == oy.keyswitch(keys, list(tensor[0]))


def test_yashe_decrypt_matches_oracle(cy):
    import torch

    n, q, t = 1024, Q127, 1024
    oy, keys, pts, cts = _setup(n, q, t)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    C = R.upload(cts)
    m = Y.decrypt(C).cpu().numpy()
    prod = Y.mul(C[:2], C[2:], relin=False)
    m2 = Y.decrypt(prod, aftermul=True).cpu().numpy()
    torch.cuda.synchronize()
    for j in range(4):
        assert [int(v) for v in m[j]] == pts[j]
    assert [int(v) for v in m2[0]] == ring.polymul_mod(pts[0], pts[2], t)
    assert [int(v) for v in m2[1]] == ring.polymul_mod(pts[1], pts[3], t)


def test_yashe_reference_suite_parameters(cy):
    """YasheSuite (src/test.cu:73-133): N = 4, t = 35951, q = the 96-bit suite
    modulus (q = 5 mod 8, so f^-1 by extended Euclid). encryptandMul decrypts
    coefficient 0 only; here every coefficient is checked."""
    import torch

    ys = GOLD["yashe_suite"]
    n, q, t = ys["degree"], int(ys["q"]), ys["t"]
    oy, keys, pts, cts = _setup(n, q, t, seed=36251)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    out = R.download(Y.mul(R.upload([cts[0]]), R.upload([cts[0]]), relin=True))
    torch.cuda.synchronize()
    assert list(out[0]) == oy.mul(keys, cts[0], cts[0], relin=True)
    assert oy.decrypt(keys, list(out[0])) == ring.polymul_mod(pts[0], pts[0], t)


def test_product_keygen_and_encrypt(cy):
    """Keys and ciphertexts made by the library decrypt correctly under the
    oracle, and the product of two of them decrypts to the plaintext product."""
    import torch

    n, q, t = 1024, Q127, 1024
    Y = cy.Yashe(n, q, t)
    Y.keygen(2024)
    F, H, EV = Y.get_keys()
    from cuyashe_gb300.api import from_limb_array

    f = [int(v) for v in from_limb_array(F)]
    # f = t f' + 1 with ternary f'
    assert all(ring.centered(v - (1 if i == 0 else 0), q) in (-t, 0, t) for i, v in enumerate(f))
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    from oracle.yashe import YasheKeys

    keys = YasheKeys(f=f, h=[int(v) for v in from_limb_array(H)],
                     evk=[[int(v) for v in row] for row in from_limb_array(EV)],
                     f2=ring.polymul_mod(f, f, q))
    rng = np.random.default_rng(5)
    m = rng.integers(0, t, size=(2, n), dtype=np.uint64)
    ct = Y.encrypt_host(m, seed=77)
    cts = [[int(v) for v in row] for row in from_limb_array(ct)]
    for j in range(2):
        assert oy.decrypt(keys, cts[j]) == [int(v) for v in m[j]]
        assert oy.noise(keys, cts[j], [int(v) for v in m[j]]) < oy.p.delta // 2**40
    R = Y.ring
    C = R.upload(ct)
    out = Y.mul(C[:1], C[1:], relin=True)
    dec = Y.decrypt(out).cpu().numpy()
    torch.cuda.synchronize()
    exp = ring.polymul_mod([int(v) for v in m[0]], [int(v) for v in m[1]], t)
    assert [int(v) for v in dec[0]] == exp
    assert list(R.download(out)[0]) == oy.mul(keys, cts[0], cts[1], relin=True)


def test_deep_level_config(cy):
    """N = 16384, q ~ 2^380 (12 digits), t = 65537: one pair, bit-exact, and
    the decryption of the product."""
    import torch

    n, q, t = 16384, Q380, 65537
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    keys = oy.keygen(9)
    smp = Sampler(10)
    m1, m2 = smp.uniform(n, t), smp.uniform(n, t)
    c1, c2 = oy.encrypt(keys, m1, 11), oy.encrypt(keys, m2, 12)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    out = Y.mul(R.upload([c1]), R.upload([c2]), relin=True)
    dec = Y.decrypt(out).cpu().numpy()
    got = R.download(out)
    torch.cuda.synchronize()
    assert [int(v) for v in dec[0]] == ring.polymul_mod(m1, m2, t)
    exp = oy.mul(keys, c1, c2, relin=True)
    assert list(got[0]) == exp
    # every N = 16384 schedule of the tensor product and the keyswitch (one-block
    # and block-pair kernels alike)
    try:
        for v in range(32):
            try:
                cy.tuning_import("n16384.l6.mulc=%d;n16384.l6.ks=%d" % (v, v))
            except cy.CyError:
                break
            got = R.download(Y.mul(R.upload([c1]), R.upload([c2]), relin=True))
            torch.cuda.synchronize()
            assert list(got[0]) == exp, "schedule %d" % v
    finally:
        cy.tuning_import("n16384.l6.mulc=0;n16384.l6.ks=0")


def test_yashe_add(cy):
    import torch

    n, q, t = 256, Q62, 257
    oy, keys, pts, cts = _setup(n, q, t)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    s = Y.add(R.upload([cts[0]]), R.upload([cts[1]]))
    dec = Y.decrypt(s).cpu().numpy()
    torch.cuda.synchronize()
    assert list(R.download(s)[0]) == oy.add(cts[0], cts[1])
    assert [int(v) for v in dec[0]] == [(x + y) % t for x, y in zip(pts[0], pts[1])]


def test_mul_without_keys_is_rejected(cy):
    n, q, t = 64, Q127, 1024
    Y = cy.Yashe(n, q, t)
    R = Y.ring
    z = R.upload([[0] * n])
    with pytest.raises(cy.CyError) as ei:
        Y.mul(z, z, relin=True)
    assert ei.value.status == -6
    Y.mul(z, z, relin=False)  # the tensor alone needs no key


@pytest.mark.parametrize("n,q,t", [(64, Q127, 1024), (512, Q190, 65537), (64, Q380, 65537)])
def test_fixed_point_rounding_equals_exact_path(cy, n, q, t):
    """The tensor epilogue estimates round(t/q x) in fixed point and falls back
    to the exact multiword path when undecided; forcing the exact path
    everywhere must give the same ciphertexts, both equal to the oracle's."""
    oy, keys, pts, cts = _setup(n, q, t)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    R = Y.ring
    A, B = R.upload([cts[0], cts[1]]), R.upload([cts[2], cts[3]])
    fast = R.download(Y.mul(A, B, relin=False))
    lib = cy.lib()
    lib.cy_set_epilogue_exact(1)
    try:
        exact = R.download(Y.mul(A, B, relin=False))
    finally:
        lib.cy_set_epilogue_exact(0)
    assert [list(x) for x in fast] == [list(x) for x in exact]
    for j in range(2):
        assert list(fast[j]) == oy.mul_tensor(cts[j], cts[2 + j])


def test_fixed_point_rounding_at_full_size(cy):
    import torch

    n, t = 4096, 1024
    Y = cy.Yashe(n, Q127, t)
    Y.keygen(17)
    rng = np.random.default_rng(17)
    m = torch.from_numpy(rng.integers(0, t, size=(256, n), dtype=np.uint64).view(np.int64)).cuda()
    c1, c2 = Y.encrypt(m, seed=1), Y.encrypt(m.flip(0).contiguous(), seed=2)
    fast = Y.mul(c1, c2, relin=False)
    lib = cy.lib()
    lib.cy_set_epilogue_exact(1)
    try:
        exact = Y.mul(c1, c2, relin=False)
    finally:
        lib.cy_set_epilogue_exact(0)
    torch.cuda.synchronize()
    assert torch.equal(fast, exact)


def _limbs_below(q, shape, rng):
    """Random coefficients in [0, q) as little-endian limbs, with q-1, (q-1)/2 and
    (q+1)/2 planted (the centring boundaries)."""
    L = (q.bit_length() + 63) // 64
    top = q.bit_length() - 64 * (L - 1) - 1
    x = rng.integers(0, 2**63, size=shape + (L,), dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    x[..., L - 1] &= np.uint64((1 << top) - 1)
    for j, v in enumerate((q - 1, (q - 1) // 2, (q + 1) // 2)):
        x[0, j] = [(v >> (64 * w)) & (2**64 - 1) for w in range(L)]
    return x


@pytest.mark.parametrize("n,q,t,kt,kr", [(4096, Q127, 1024, 9, 6), (2048, Q62, 65537, 5, 4),
                                         (8192, Q190, 65537, 14, 8), (16384, Q380, 65537, 26, 15)])
def test_specialised_epilogues_equal_generic(cy, n, q, t, kt, kr):
    """The epilogues compiled for these prime counts (constants passed by value)
    give the generic kernel's results bit for bit: tensor rounding, keyswitch and
    plain product."""
    import torch

    Y = cy.Yashe(n, q, t)
    Y.keygen(3)
    info = Y.info()
    assert (info.tensor_primes, info.relin_primes) == (kt, kr)
    batch = 64 if n <= 4096 else 6
    rng = np.random.default_rng(n)
    C1 = torch.from_numpy(_limbs_below(q, (batch, n), rng).view(np.int64)).cuda()
    C2 = torch.from_numpy(_limbs_below(q, (batch, n), rng).view(np.int64)).cuda()
    P = cy.Ring(n, q)
    lib = cy.lib()
    outs = []
    for generic in (0, 1):
        lib.cy_set_epilogue_generic(generic)
        try:
            outs.append((Y.mul(C1, C2, relin=False), Y.mul(C1, C2, relin=True), P.polymul(C1, C2)))
            torch.cuda.synchronize()
        finally:
            lib.cy_set_epilogue_generic(0)
    for a, b in zip(*outs):
        assert torch.equal(a, b)
    # and the oracle's tensor product for the first pair at N <= 4096
    if n <= 4096:
        oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
        to_int = lambda a: [sum(int(a[i, w]) << (64 * w) for w in range(a.shape[1])) for i in range(n)]
        h1, h2 = C1[0].cpu().numpy().view(np.uint64), C2[0].cpu().numpy().view(np.uint64)
        got = outs[0][0][0].cpu().numpy().view(np.uint64)
        assert to_int(got) == oy.mul_tensor(to_int(h1), to_int(h2))
