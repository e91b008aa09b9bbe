"""Wire / on-disk format of keys and ciphertexts (cy_serialize & co., host only).

The layout is pinned by an independent encoder written here with `struct`
from the format's description (include/cuyashe.h): the library's bytes must
equal it. Corrupted, truncated or foreign blobs must be refused.
"""
import struct

import numpy as np
import pytest

from cuyashe_gb300 import CyError
from cuyashe_gb300 import api

Q127 = 2**127 - 1
Q190 = 1569275433846670190958947355801916604025588861116000698369


def _fnv1a(data: bytes) -> int:
    h = 0xCBF29CE484222325
    for b in data:
        h = ((h ^ b) * 0x100000001B3) & (2**64 - 1)
    return h


def _encode(kind, n, q, L, t, w_bits, polys):
    out = b"CYSH" + struct.pack("<IIIIIQII", 1, kind, n, L, polys.shape[0], t, w_bits, 0)
    out += b"".join(struct.pack("<Q", (q >> (64 * i)) & (2**64 - 1)) for i in range(L))
    out += polys.astype("<u8").tobytes()
    return out + struct.pack("<Q", _fnv1a(out))


def _rand(rng, count, n, q, L):
    vals = [[int(rng.integers(0, 2**62)) * int(rng.integers(1, 2**62)) % q for _ in range(n)] for _ in range(count)]
    return np.array([[[(v >> (64 * w)) & (2**64 - 1) for w in range(L)] for v in p] for p in vals], dtype=np.uint64)


@pytest.mark.parametrize("q,L", [(Q127, 2), (Q190, 3)])
def test_layout_matches_independent_encoder(q, L):
    rng = np.random.default_rng(L)
    polys = _rand(rng, 3, 16, q, L)
    blob = api.serialize(1, 16, q, polys, t=1024, w_bits=32)
    assert blob == _encode(1, 16, q, L, 1024, 32, polys)
    info, back = api.deserialize(blob)
    assert info == {"kind": 1, "n": 16, "q": q, "q_limbs": L, "count": 3, "t": 1024, "w_bits": 32,
                    "bytes": len(blob)}
    assert np.array_equal(back, polys)


def test_empty_blob_and_size_query():
    blob = api.serialize(1, 8, Q127, np.zeros((0, 8, 2), np.uint64))
    info, back = api.deserialize(blob)
    assert info["count"] == 0 and back.shape == (0, 8, 2)
    assert len(blob) == 40 + 16 + 8


def test_corruption_is_detected():
    polys = _rand(np.random.default_rng(1), 2, 8, Q127, 2)
    blob = api.serialize(2, 8, Q127, polys)
    for pos in (0, 4, 9, 13, 20, 30, 45, 100, len(blob) - 1):
        bad = bytearray(blob)
        bad[pos] ^= 0x40
        with pytest.raises(CyError):
            api.deserialize(bytes(bad))
    for cut in (0, 10, 39, len(blob) - 1):
        with pytest.raises(CyError):
            api.deserialize(blob[:cut])


def test_bad_inputs_are_refused():
    polys = _rand(np.random.default_rng(2), 1, 8, Q127, 2)
    over = polys.copy()
    over[0, 3] = [2**64 - 1, 2**63 - 1]  # = q
    with pytest.raises(CyError):
        api.serialize(1, 8, Q127, over)
    with pytest.raises(CyError):
        api.serialize(9, 8, Q127, polys)  # unknown kind
    # a blob whose coefficients were edited past q with a recomputed checksum
    raw = bytearray(_encode(1, 8, Q127, 2, 0, 0, polys)[:-8])
    raw[40 + 16: 40 + 32] = struct.pack("<QQ", 2**64 - 1, 2**63 - 1)
    forged = bytes(raw) + struct.pack("<Q", _fnv1a(bytes(raw)))
    with pytest.raises(CyError):
        api.deserialize(forged)


@pytest.mark.gpu
def test_keys_save_and_resume():
    import torch

    import cuyashe_gb300 as cy

    n, q, t = 1024, 170141183460469231731687303715883253761, 1024
    Y1 = cy.Yashe(n, q, t)
    Y1.keygen(31)
    blob = Y1.save_keys()
    info = api.blob_info(blob)
    assert info["kind"] == cy.BLOB_KEYS and info["count"] == 2 + Y1.ell and info["t"] == t
    Y2 = cy.Yashe(n, q, t)
    Y2.load_keys(blob)
    F1, H1, E1 = Y1.get_keys()
    F2, H2, E2 = Y2.get_keys()
    assert np.array_equal(F1, F2) and np.array_equal(H1, H2) and np.array_equal(E1, E2)
    m = torch.from_numpy(np.random.default_rng(3).integers(0, t, size=(8, n), dtype=np.uint64).view(np.int64)).cuda()
    c = Y1.encrypt(m, seed=4)
    assert torch.equal(Y2.encrypt(m, seed=4), c)
    assert torch.equal(Y1.mul(c, c), Y2.mul(c, c))
    with pytest.raises(CyError):
        cy.Yashe(n, q, 257).load_keys(blob)  # other t
    bad = bytearray(blob)
    bad[100] ^= 1
    with pytest.raises(CyError):
        Y2.load_keys(bytes(bad))
