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


def _words(vals, L):
    return [[(v >> (64 * w)) & (2**64 - 1) for w in range(L)] for v in vals]


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
