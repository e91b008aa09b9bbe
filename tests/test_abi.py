"""The C-ABI library loads and exports every symbol include/cuyashe.h declares (CPU).

No compute calls here: only symbol presence, status strings, and argument
validation paths that return before touching the GPU.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "cuyashe.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cy_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def L():
    from cuyashe_gb300 import build

    build.build()
    import cuyashe_gb300

    return cuyashe_gb300.lib()


def test_header_declares_entry_points():
    names = _declared()
    for required in ["cy_ring_create", "cy_polymul", "cy_yashe_mul", "cy_yashe_keyswitch", "cy_yashe_decrypt",
                     "cy_ntt", "cy_crt", "cy_icrt", "cy_polymul_batched"]:
        assert required in names


def test_every_declared_symbol_is_exported(L):
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    import cuyashe_gb300

    assert set(_declared()) == set(cuyashe_gb300.SIGNATURES)


def test_status_strings(L):
    assert L.cy_status_string(0) == b"ok"
    assert L.cy_status_string(-1) == b"invalid argument"
    assert L.cy_status_string(12345) == b"unknown status"
    assert L.cy_version() >= 1


def test_null_arguments_rejected_without_gpu(L):
    h = ctypes.c_void_p()
    assert L.cy_ring_create(8, None, 2, ctypes.byref(h)) == -1
    assert L.cy_ring_destroy(None) == 0
    assert L.cy_polymul(None, None, None, None, 1, None) == -1
    assert L.cy_yashe_mul(None, None, None, None, 1, 1, None) == -1
    assert b"NULL" in L.cy_last_error() or b"null" in L.cy_last_error().lower()


def test_bad_sizes_rejected_without_gpu(L):
    import cuyashe_gb300 as cy

    h = ctypes.c_void_p()
    q = cy.limbs_of(2**127 - 1, 2)
    assert L.cy_ring_create(12, q, 2, ctypes.byref(h)) == -2  # not a power of two
    assert L.cy_ring_create(1 << 15, q, 2, ctypes.byref(h)) == -2  # beyond 16384
    assert L.cy_ring_create(8, q, 7, ctypes.byref(h)) == -2  # q wider than 384 bits
