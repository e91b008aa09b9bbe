"""cuyashe_gb300 -- GB300-native (sm_103a) hot path of cuYASHE behind a C ABI.

The product is ``libcuyashe_gb300.so`` (CUDA kernels + ``extern "C"`` entry
points declared in ``include/cuyashe.h``). This package loads it with ctypes
and offers a thin Python mirror of the reference's objects (``Ring`` for
``Polynomial`` arithmetic in Z_q[x]/(x^N+1), ``Yashe`` for the scheme) so that
tests and the benchmark call exactly the C ABI a C/C++ host would call.

Device buffers are torch CUDA tensors (uint64 / int64 storage); torch is used
only for memory and streams. There is no CPU fallback: importing works without
a GPU (for ABI checks), every compute call needs the CUDA library and a GPU.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcuyashe_gb300.so")

CY_OK = 0
STATUS = {
    0: "CY_OK",
    -1: "CY_ERR_INVALID_ARGUMENT",
    -2: "CY_ERR_UNSUPPORTED",
    -3: "CY_ERR_CUDA",
    -4: "CY_ERR_OUT_OF_MEMORY",
    -5: "CY_ERR_NOT_INVERTIBLE",
    -6: "CY_ERR_NO_KEYS",
    -7: "CY_ERR_TIMEOUT",
    -8: "CY_ERR_BUSY",
    -9: "CY_ERR_INTERNAL",
}

MAX_CRT_PRIMES = 40


class CyError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__("%s failed: %s (%s)" % (where, STATUS.get(status, status), msg))
        self.status = status


class RingInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("q_limbs", ctypes.c_int), ("q_bits", ctypes.c_int),
                ("crt_primes", ctypes.c_int), ("crt_bits", ctypes.c_int),
                ("primes", ctypes.c_uint32 * MAX_CRT_PRIMES)]


class YasheParams(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("q", ctypes.POINTER(ctypes.c_uint64)), ("q_limbs", ctypes.c_int),
                ("t", ctypes.c_uint64), ("w_bits", ctypes.c_int), ("sigma", ctypes.c_double)]


class YasheInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("q_limbs", ctypes.c_int), ("q_bits", ctypes.c_int), ("ell", ctypes.c_int),
                ("w_bits", ctypes.c_int), ("t", ctypes.c_uint64), ("tensor_primes", ctypes.c_int),
                ("relin_primes", ctypes.c_int), ("has_keys", ctypes.c_int)]


class TraceEntry(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_int), ("total_ms", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device_budget_bytes", ctypes.c_size_t), ("streams", ctypes.c_int), ("max_batch", ctypes.c_int),
                ("poll_us", ctypes.c_int), ("batch_budget_us", ctypes.c_int)]


class ServeRequest(ctypes.Structure):
    _fields_ = [("class_id", ctypes.c_int), ("relin", ctypes.c_int), ("h_c1", ctypes.c_void_p),
                ("h_c2", ctypes.c_void_p), ("h_out", ctypes.c_void_p)]


class ServeRequestDev(ctypes.Structure):
    _fields_ = [("class_id", ctypes.c_int), ("relin", ctypes.c_int), ("d_c1", ctypes.c_void_p),
                ("d_c2", ctypes.c_void_p), ("d_out", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("rejected", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double),
                ("mean_us", ctypes.c_double), ("throughput_per_s", ctypes.c_double),
                ("peak_device_bytes", ctypes.c_size_t)]


class BlobInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("n", ctypes.c_int), ("q_limbs", ctypes.c_int), ("count", ctypes.c_int),
                ("w_bits", ctypes.c_int), ("t", ctypes.c_uint64), ("q", ctypes.c_uint64 * 12),
                ("bytes", ctypes.c_size_t)]


BLOB_CIPHERTEXTS, BLOB_PUBLIC_KEY, BLOB_SECRET_KEY, BLOB_EVAL_KEY, BLOB_KEYS = 1, 2, 3, 4, 5


class PolymulJob(ctypes.Structure):
    _fields_ = [("ring", ctypes.c_void_p), ("d_a", ctypes.c_void_p), ("d_b", ctypes.c_void_p),
                ("d_c", ctypes.c_void_p)]


class MixedJobC(ctypes.Structure):
    _fields_ = [("ring", ctypes.c_void_p), ("yashe", ctypes.c_void_p), ("relin", ctypes.c_int),
                ("d_a", ctypes.c_void_p), ("d_b", ctypes.c_void_p), ("d_c", ctypes.c_void_p)]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_u64p = ctypes.POINTER(ctypes.c_uint64)

# name -> argtypes (all return int cy_status unless noted)
SIGNATURES = {
    "cy_status_string": ([_i], ctypes.c_char_p),
    "cy_last_error": ([], ctypes.c_char_p),
    "cy_version": ([], _i),
    "cy_ring_create": ([_i, _u64p, _i, ctypes.POINTER(_vp)], _i),
    "cy_ring_destroy": ([_vp], _i),
    "cy_ring_get_info": ([_vp, ctypes.POINTER(RingInfo)], _i),
    "cy_workspace_create": ([ctypes.POINTER(_vp)], _i),
    "cy_workspace_destroy": ([_vp], _i),
    "cy_polymul": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_polymul_ws": ([_vp, _vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_polymul_host": ([_vp, _vp, _vp, _vp, _i], _i),
    "cy_polyadd": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_polysub": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_poly_scalar_mul": ([_vp, _vp, _u64p, _vp, _i, _vp], _i),
    "cy_polymul_batched": ([ctypes.POINTER(PolymulJob), _i, _vp], _i),
    "cy_polymul_noalloc": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_polymul_batched_status": ([_vp], _i),
    "cy_mixed_plan_create": ([ctypes.POINTER(MixedJobC), _i, ctypes.POINTER(_vp)], _i),
    "cy_mixed_plan_destroy": ([_vp], _i),
    "cy_mixed_plan_launch": ([_vp, _vp], _i),
    "cy_mixed_plan_status": ([_vp, _vp], _i),
    "cy_mixed_plan_set_schedule": ([_vp, _i], _i),
    "cy_mixed_plan_get_schedule": ([_vp, ctypes.POINTER(_i)], _i),
    "cy_mixed_plan_autotune": ([_vp, _vp], _i),
    "cy_mixed_plan_test_starve": ([_vp, _i, ctypes.c_uint], _i),
    "cy_mixed_plan_graph_create": ([_vp, ctypes.POINTER(_vp)], _i),
    "cy_ntt": ([_vp, _vp, _i, _i, _vp], _i),
    "cy_ntt_check": ([], _i),
    "cy_ntt_test_wait": ([ctypes.c_uint, ctypes.c_uint], _i),
    "cy_crt": ([_vp, _vp, _vp, _i, _vp], _i),
    "cy_icrt": ([_vp, _vp, _vp, _i, _vp], _i),
    "cy_yashe_create": ([ctypes.POINTER(YasheParams), ctypes.POINTER(_vp)], _i),
    "cy_yashe_destroy": ([_vp], _i),
    "cy_yashe_get_info": ([_vp, ctypes.POINTER(YasheInfo)], _i),
    "cy_yashe_get_ring": ([_vp, ctypes.POINTER(_vp)], _i),
    "cy_yashe_keygen": ([_vp, ctypes.c_uint64], _i),
    "cy_yashe_set_keys": ([_vp, _vp, _vp, _vp], _i),
    "cy_yashe_get_keys": ([_vp, _vp, _vp, _vp], _i),
    "cy_yashe_encrypt_host": ([_vp, _vp, _vp, _i, ctypes.c_uint64], _i),
    "cy_yashe_decrypt": ([_vp, _vp, _vp, _i, _i, _vp], _i),
    "cy_yashe_mul": ([_vp, _vp, _vp, _vp, _i, _i, _vp], _i),
    "cy_yashe_mul_ws": ([_vp, _vp, _vp, _vp, _vp, _i, _i, _vp], _i),
    "cy_yashe_mul_host": ([_vp, _vp, _vp, _vp, _i, _i], _i),
    "cy_yashe_encrypt": ([_vp, _vp, _vp, _i, ctypes.c_uint64, _vp], _i),
    "cy_gaussian_cdt": ([ctypes.c_double, _u64p, _i, ctypes.POINTER(_i)], _i),
    "cy_serialize": ([ctypes.c_uint32, _i, _vp, _i, ctypes.c_uint64, _i, _vp, _i, _vp, ctypes.c_size_t,
                      ctypes.POINTER(ctypes.c_size_t)], _i),
    "cy_blob_info_read": ([_vp, ctypes.c_size_t, ctypes.POINTER(BlobInfo)], _i),
    "cy_deserialize": ([_vp, ctypes.c_size_t, _vp, ctypes.c_size_t], _i),
    "cy_yashe_save_keys": ([_vp, _vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], _i),
    "cy_yashe_load_keys": ([_vp, _vp, ctypes.c_size_t], _i),
    "cy_yashe_keyswitch": ([_vp, _vp, _vp, _i, _vp], _i),
    "cy_yashe_add": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_yashe_add_plain": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_yashe_mul_plain": ([_vp, _vp, _vp, _vp, _i, _vp], _i),
    "cy_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)], _i),
    "cy_server_destroy": ([_vp], _i),
    "cy_server_register": ([_vp, _vp, ctypes.POINTER(_i)], _i),
    "cy_server_submit": ([_vp, ctypes.POINTER(ServeRequest), ctypes.POINTER(ctypes.c_uint64)], _i),
    "cy_server_submit_device": ([_vp, ctypes.POINTER(ServeRequestDev), _i, ctypes.POINTER(ctypes.c_uint64)], _i),
    "cy_server_poll": ([_vp, ctypes.c_uint64, ctypes.POINTER(_i)], _i),
    "cy_server_wait": ([_vp, ctypes.c_uint64, _i], _i),
    "cy_server_drain": ([_vp, _i], _i),
    "cy_server_get_stats": ([_vp, ctypes.POINTER(ServerStats)], _i),
    "cy_server_reset_stats": ([_vp], _i),
    "cy_polymul_graph_create": ([_vp, _vp, _vp, _vp, _i, ctypes.POINTER(_vp)], _i),
    "cy_yashe_mul_graph_create": ([_vp, _vp, _vp, _vp, _i, _i, ctypes.POINTER(_vp)], _i),
    "cy_graph_launch": ([_vp, _vp], _i),
    "cy_graph_destroy": ([_vp], _i),
    "cy_ring_autotune": ([_vp, _i, _vp], _i),
    "cy_yashe_autotune": ([_vp, _i, _vp], _i),
    "cy_tuning_export": ([ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], _i),
    "cy_tuning_import": ([ctypes.c_char_p], _i),
    "cy_set_epilogue_exact": ([_i], _i),
    "cy_set_epilogue_generic": ([_i], _i),
    "cy_set_chunk_overlap": ([_i], _i),
    "cy_launch_count": ([], ctypes.c_uint64),
    "cy_trace_start": ([], _i),
    "cy_trace_stop": ([ctypes.POINTER(TraceEntry), _i, ctypes.POINTER(_i)], _i),
}

_lib = None


def lib(build_if_missing: bool = False):
    """The loaded C library. Raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _b
            _b.build()
        else:
            raise ImportError("libcuyashe_gb300.so is not built; run `python -m cuyashe_gb300.build` "
                              "(the GPU path has no fallback)")
    L = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(status: int, where: str) -> None:
    if status != CY_OK:
        msg = lib().cy_last_error()
        raise CyError(status, where, msg.decode() if msg else "")


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _ptr(t) -> int:
    return t.data_ptr() if t is not None else 0


def limbs_of(x: int, n: int):
    return (ctypes.c_uint64 * n)(*[(x >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(n)])


def tuning_export() -> str:
    """The autotuner's choices for the current device ("n4096.l2.mul=1;...")."""
    need = ctypes.c_size_t(0)
    check(lib().cy_tuning_export(None, 0, ctypes.byref(need)), "cy_tuning_export")
    buf = ctypes.create_string_buffer(need.value + 1)
    check(lib().cy_tuning_export(buf, len(buf), ctypes.byref(need)), "cy_tuning_export")
    return buf.value.decode()


def tuning_import(spec: str) -> None:
    check(lib().cy_tuning_import(spec.encode()), "cy_tuning_import")


def launch_count() -> int:
    """Kernels launched by the library so far."""
    return int(lib().cy_launch_count())


class Trace:
    """Context manager: per-kernel launch counts and device time (CUDA events)."""

    def __enter__(self):
        check(lib().cy_trace_start(), "cy_trace_start")
        self.kernels = {}
        return self

    def __exit__(self, *exc):
        buf = (TraceEntry * 256)()
        n = ctypes.c_int(0)
        check(lib().cy_trace_stop(buf, 256, ctypes.byref(n)), "cy_trace_stop")
        self.kernels = {buf[i].name.decode(): (buf[i].launches, buf[i].total_ms) for i in range(min(n.value, 256))}
        return False


from .api import MixedPlan, Ring, Yashe, Workspace  # noqa: E402,F401
