"""GPU encryption with on-device sampling (cy_yashe_encrypt) against the oracle.

Every ciphertext must equal the oracle's [h*s + e + Delta*(m mod t)]_q with s
and e drawn by the oracle's restatement of the counter-based sampler, bit for
bit; GPU decryption must return m; encrypt -> multiply -> decrypt must give
m1*m2 mod t entirely on the GPU.
"""
import random

import numpy as np
import pytest

from oracle import ring, sampling
from oracle.yashe import Yashe as OYashe
from oracle.yashe import YasheParams

pytestmark = pytest.mark.gpu

QY = 170141183460469231731687303715883253761  # largest prime < 2^127 with q = 1 mod 2^16


@pytest.fixture(scope="module")
def cy():
    import torch

    import cuyashe_gb300

    assert torch.cuda.is_available()
    cuyashe_gb300.lib()
    return cuyashe_gb300


@pytest.mark.parametrize("n,qbits,t", [(64, 127, 257), (256, 62, 65537), (1024, 190, 1024)])
def test_encrypt_matches_oracle(cy, n, qbits, t):
    import torch

    q = ring.largest_prime_below(2**qbits, congruent_mod=2 * n)
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    keys = oy.keygen(n + 3)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    batch, seed = 3, 0x1234567 + n
    rng = random.Random(n)
    m = [[rng.randrange(t) for _ in range(n)] for _ in range(batch)]
    m[1][0] = t + 5  # taken mod t
    dm = torch.tensor(np.array(m, dtype=np.uint64).view(np.int64), device="cuda")
    ct = Y.ring.download(Y.encrypt(dm, seed))
    s, e = sampling.encryption_errors(seed, batch, n, 8.0)
    for b in range(batch):
        want = oy.encrypt_with_errors(keys, m[b], s[b], e[b])
        assert list(ct[b]) == want
        assert oy.decrypt(keys, want) == [v % t for v in m[b]]


def test_encrypt_decrypt_and_multiply_on_gpu(cy):
    import torch

    n, t, batch = 4096, 1024, 64
    Y = cy.Yashe(n, QY, t)
    Y.keygen(99)
    rng = np.random.default_rng(4)
    m1 = rng.integers(0, t, size=(batch, n), dtype=np.uint64)
    m2 = rng.integers(0, t, size=(batch, n), dtype=np.uint64)
    d1 = torch.from_numpy(m1.view(np.int64)).cuda()
    d2 = torch.from_numpy(m2.view(np.int64)).cuda()
    c1 = Y.encrypt(d1, seed=1)
    c2 = Y.encrypt(d2, seed=2)
    assert np.array_equal(Y.decrypt(c1).cpu().numpy().view(np.uint64), m1)
    prod = Y.mul(c1, c2, relin=True)
    got = Y.decrypt(prod).cpu().numpy().view(np.uint64)
    PT = cy.Ring(n, t)
    want = PT.polymul(PT.upload(m1[:4].astype(object).tolist()), PT.upload(m2[:4].astype(object).tolist()))
    assert np.array_equal(got[:4], want.cpu().numpy().view(np.uint64)[..., 0])
    # same seed, same ciphertexts; another seed, others
    assert torch.equal(Y.encrypt(d1, seed=1), c1)
    assert not torch.equal(Y.encrypt(d1, seed=3), c1)


def test_encrypt_one_ciphertext_at_full_size_matches_oracle(cy):
    import torch

    n, t = 4096, 1024
    Y = cy.Yashe(n, QY, t)
    Y.keygen(5)
    F, H, EV = Y.get_keys()
    L = Y.ring.L
    to_int = lambda a: [sum(int(a[i, w]) << (64 * w) for w in range(L)) for i in range(n)]
    oy = OYashe(YasheParams(n=n, q=QY, t=t, w_bits=32))
    from oracle.yashe import YasheKeys
    keys = YasheKeys(f=to_int(F), h=to_int(H), evk=[to_int(EV[d]) for d in range(EV.shape[0])])
    m = list(np.random.default_rng(8).integers(0, t, size=n))
    dm = torch.tensor(np.array([m], dtype=np.uint64).view(np.int64), device="cuda")
    ct = Y.ring.download(Y.encrypt(dm, seed=77))[0]
    s, e = sampling.encryption_errors(77, 1, n, 8.0)
    assert list(ct) == oy.encrypt_with_errors(keys, m, s[0], e[0])


def test_encrypt_rejects_bad_arguments(cy):
    import torch

    Y = cy.Yashe(64, ring.largest_prime_below(2**127, congruent_mod=128), 257)
    m = torch.zeros((1, 64), dtype=torch.int64, device="cuda")
    ct = Y.ring.empty(1)
    lib = cy.lib()
    assert lib.cy_yashe_encrypt(Y.h, m.data_ptr(), ct.data_ptr(), 1, 1, None) == -6  # no keys
    Y.keygen(1)
    assert lib.cy_yashe_encrypt(Y.h, m.data_ptr(), ct.data_ptr(), 0, 1, None) == 0
    assert lib.cy_yashe_encrypt(Y.h, 0, ct.data_ptr(), 1, 1, None) == -1
    assert lib.cy_yashe_encrypt(Y.h, m.data_ptr(), ct.data_ptr() + 8, 1, 1, None) == -1  # misaligned
    assert lib.cy_yashe_encrypt(None, m.data_ptr(), ct.data_ptr(), 1, 1, None) == -1


@pytest.mark.parametrize("n,qbits,t", [(64, 127, 257), (256, 190, 65537)])
def test_plaintext_ops_match_oracle(cy, n, qbits, t):
    import torch

    q = ring.largest_prime_below(2**qbits, congruent_mod=2 * n)
    oy = OYashe(YasheParams(n=n, q=q, t=t, w_bits=32))
    keys = oy.keygen(n + 11)
    Y = cy.Yashe(n, q, t)
    Y.set_keys(keys.f, keys.h, keys.evk)
    rng = random.Random(n + 1)
    m1 = [[rng.randrange(t) for _ in range(n)] for _ in range(2)]
    m2 = [[rng.randrange(2 * t) for _ in range(n)] for _ in range(2)]  # taken mod t
    cts = [oy.encrypt(keys, m, 50 + i) for i, m in enumerate(m1)]
    C = Y.ring.upload(cts)
    M2 = torch.tensor(np.array(m2, dtype=np.uint64).view(np.int64), device="cuda")
    add = Y.ring.download(Y.add_plain(C, M2))
    mul = Y.ring.download(Y.mul_plain(C, M2))
    for j in range(2):
        assert list(add[j]) == oy.add_plain(cts[j], m2[j])
        assert list(mul[j]) == oy.mul_plain(cts[j], m2[j])
        m2t = [v % t for v in m2[j]]
        assert oy.decrypt(keys, list(add[j])) == [(a + b) % t for a, b in zip(m1[j], m2t)]
        assert oy.decrypt(keys, list(mul[j])) == ring.polymul_mod(m1[j], m2t, t)


def test_plaintext_ops_decrypt_at_full_size(cy):
    import torch

    n, t, batch = 4096, 1024, 16
    Y = cy.Yashe(n, QY, t)
    Y.keygen(12)
    rng = np.random.default_rng(6)
    m1 = rng.integers(0, t, size=(batch, n), dtype=np.uint64)
    m2 = rng.integers(0, t, size=(batch, n), dtype=np.uint64)
    d1 = torch.from_numpy(m1.view(np.int64)).cuda()
    d2 = torch.from_numpy(m2.view(np.int64)).cuda()
    c = Y.encrypt(d1, seed=21)
    got_add = Y.decrypt(Y.add_plain(c, d2)).cpu().numpy().view(np.uint64)
    assert np.array_equal(got_add, (m1 + m2) % t)
    got_mul = Y.decrypt(Y.mul_plain(c, d2)).cpu().numpy().view(np.uint64)
    PT = cy.Ring(n, t)
    want = PT.polymul(PT.upload(m1[:2].astype(object).tolist()), PT.upload(m2[:2].astype(object).tolist()))
    assert np.array_equal(got_mul[:2], want.cpu().numpy().view(np.uint64)[..., 0])
    lib = cy.lib()
    assert lib.cy_yashe_mul_plain(Y.h, c.data_ptr(), d2.data_ptr(), c.data_ptr(), batch, None) == -1  # aliasing
