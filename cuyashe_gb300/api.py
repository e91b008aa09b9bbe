"""Python mirror of the reference's host objects over the C ABI.

``Ring``  ~ the reference's ``Polynomial`` arithmetic for one (N, q):
            ``polymul`` = ``Polynomial c = a*b; c.reduce();`` (src/polynomial.cpp:52-60,
            src/cuda_functions.cu:1040-1077), ``polyadd``/``polysub`` =
            ``operator+``/``operator-`` followed by ``% q``, ``scalar_mul`` =
            ``operator*(ZZ)`` (src/polynomial.h:533-573).
``Yashe`` ~ ``Yashe`` + ``Ciphertext`` (src/yashe.h, src/ciphertext.h):
            ``keygen``, ``encrypt``, ``decrypt``, ``mul`` (``Ciphertext::operator*``,
            optionally followed by ``convert``), ``keyswitch`` (``convert``), ``add``.

Polynomials are [batch][N][L] little-endian uint64 limbs. On the device they are
torch int64 tensors holding the same bits; on the host numpy uint64 arrays.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import (CY_OK, BLOB_KEYS, BlobInfo, MixedJobC, PolymulJob, RingInfo, ServeRequest, ServeRequestDev, ServerConfig, ServerStats, YasheInfo, YasheParams, _ptr,
               _stream_handle, check, lib, limbs_of)


def nlimbs(q: int) -> int:
    return max(1, ((q - 1).bit_length() + 63) // 64)


def to_limb_array(values, L: int) -> np.ndarray:
    """ints (nested lists ok) -> uint64 array with a trailing limb axis."""
    arr = np.asarray(values, dtype=object)
    flat = arr.reshape(-1)
    raw = b"".join(int(v).to_bytes(8 * L, "little") for v in flat)
    return np.frombuffer(raw, dtype="<u8").reshape(arr.shape + (L,)).copy()


def from_limb_array(arr: np.ndarray):
    a = np.ascontiguousarray(arr, dtype="<u8")
    L = a.shape[-1]
    flat = a.reshape(-1, L)
    raw = flat.tobytes()
    vals = [int.from_bytes(raw[i * 8 * L:(i + 1) * 8 * L], "little") for i in range(flat.shape[0])]
    return np.array(vals, dtype=object).reshape(a.shape[:-1])


def _host_ptr(x) -> int:
    """Address of a C-contiguous host array of 8-byte words: a numpy array, or a
    CPU torch tensor (page-locked ones let the copies overlap the kernels)."""
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous or x.dtype.itemsize != 8:
            raise ValueError("host arrays must be C-contiguous with 8-byte elements")
        return x.ctypes.data
    if x.device.type != "cpu" or not x.is_contiguous() or x.element_size() != 8:
        raise ValueError("host tensors must be contiguous CPU tensors with 8-byte elements")
    return x.data_ptr()


def serialize(kind: int, n: int, q: int, polys: np.ndarray, t: int = 0, w_bits: int = 0) -> bytes:
    """Blob (cy_serialize) of polynomials [count][n][L] uint64 limbs mod q."""
    L = nlimbs(q)
    polys = np.ascontiguousarray(polys, dtype=np.uint64).reshape(-1, n, L)
    qa = np.array([(q >> (64 * i)) & (2**64 - 1) for i in range(L)], dtype=np.uint64)
    need = ctypes.c_size_t(0)
    check(lib().cy_serialize(kind, n, qa.ctypes.data, L, t, w_bits, polys.ctypes.data, polys.shape[0], None, 0,
                             ctypes.byref(need)), "cy_serialize")
    buf = ctypes.create_string_buffer(need.value)
    check(lib().cy_serialize(kind, n, qa.ctypes.data, L, t, w_bits, polys.ctypes.data, polys.shape[0], buf,
                             need.value, ctypes.byref(need)), "cy_serialize")
    return buf.raw


def blob_info(blob: bytes) -> dict:
    info = BlobInfo()
    check(lib().cy_blob_info_read(blob, len(blob), ctypes.byref(info)), "cy_blob_info_read")
    q = sum(int(info.q[i]) << (64 * i) for i in range(info.q_limbs))
    return {"kind": info.kind, "n": info.n, "q": q, "q_limbs": info.q_limbs, "count": info.count, "t": info.t,
            "w_bits": info.w_bits, "bytes": info.bytes}


def deserialize(blob: bytes):
    """(header dict, polynomials [count][n][L] uint64) of a checked blob."""
    info = blob_info(blob)
    out = np.zeros((info["count"], info["n"], info["q_limbs"]), np.uint64)
    check(lib().cy_deserialize(blob, len(blob), out.ctypes.data, out.size), "cy_deserialize")
    return info, out


def to_device(arr: np.ndarray, device="cuda"):
    import torch
    a = np.ascontiguousarray(arr, dtype=np.uint64)
    return torch.from_numpy(a.view(np.int64)).to(device)


def to_host(t) -> np.ndarray:
    return t.detach().cpu().numpy().view(np.uint64)


class Workspace:
    """Scratch for calls issued on different streams at the same time."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().cy_workspace_create(ctypes.byref(h)), "cy_workspace_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().cy_workspace_destroy(self.h)
            self.h = None


class Graph:
    """A fixed batch recorded as a CUDA graph (``cy_*_graph_create``); keeps its
    buffers alive and replays with ``launch``."""

    def __init__(self, handle: ctypes.c_void_p, keep):
        self.h, self._keep = handle, keep

    def launch(self, stream=None) -> None:
        check(lib().cy_graph_launch(self.h, _stream_handle(stream)), "cy_graph_launch")

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().cy_graph_destroy(self.h)
            self.h = ctypes.c_void_p()


class Ring:
    """Z_q[x]/(x^N+1) on the GPU (handle to a ``cy_ring``)."""

    def __init__(self, n: int, q: int, handle: Optional[ctypes.c_void_p] = None, owner=None):
        self.n, self.q, self.L = n, q, nlimbs(q)
        self._owner = owner
        if handle is None:
            h = ctypes.c_void_p()
            check(lib().cy_ring_create(n, limbs_of(q, self.L), self.L, ctypes.byref(h)), "cy_ring_create")
            self.h, self._own = h, True
        else:
            self.h, self._own = handle, False
        info = RingInfo()
        check(lib().cy_ring_get_info(self.h, ctypes.byref(info)), "cy_ring_get_info")
        self.info = info
        self.k = info.crt_primes
        self.primes = [info.primes[i] for i in range(info.crt_primes)]

    def __del__(self):
        if getattr(self, "_own", False) and self.h.value:
            lib().cy_ring_destroy(self.h)
            self.h = ctypes.c_void_p()

    # -- buffers ----------------------------------------------------------
    def empty(self, batch: int, device="cuda"):
        import torch
        return torch.empty((batch, self.n, self.L), dtype=torch.int64, device=device)

    def upload(self, polys) -> "torch.Tensor":  # noqa: F821
        """list of polynomials (lists of ints in [0, q)) or a limb array -> device tensor."""
        arr = polys if isinstance(polys, np.ndarray) and polys.dtype == np.uint64 else to_limb_array(polys, self.L)
        if arr.ndim == 2:
            arr = arr[None]
        return to_device(arr)

    def download(self, t):
        return from_limb_array(to_host(t))

    # -- ops ----------------------------------------------------------------
    def polymul(self, a, b, out=None, stream=None, workspace: Optional[Workspace] = None):
        batch = a.shape[0]
        out = self.empty(batch) if out is None else out
        st = _stream_handle(stream)
        if workspace is None:
            check(lib().cy_polymul(self.h, _ptr(a), _ptr(b), _ptr(out), batch, st), "cy_polymul")
        else:
            check(lib().cy_polymul_ws(self.h, workspace.h, _ptr(a), _ptr(b), _ptr(out), batch, st), "cy_polymul_ws")
        return out

    def polymul_host(self, a, b, out=None):
        """a*b with a, b, out in host memory ([batch][N][L] words: numpy arrays or
        CPU torch tensors)."""
        if isinstance(a, np.ndarray):
            a = np.ascontiguousarray(a, dtype=np.uint64)
            b = np.ascontiguousarray(b, dtype=np.uint64)
        out = (np.empty_like(a) if isinstance(a, np.ndarray) else a.new_empty(a.shape)) if out is None else out
        check(lib().cy_polymul_host(self.h, _host_ptr(a), _host_ptr(b), _host_ptr(out), a.shape[0]),
              "cy_polymul_host")
        return out

    def polyadd(self, a, b, out=None, stream=None):
        out = self.empty(a.shape[0]) if out is None else out
        check(lib().cy_polyadd(self.h, _ptr(a), _ptr(b), _ptr(out), a.shape[0], _stream_handle(stream)),
              "cy_polyadd")
        return out

    def polysub(self, a, b, out=None, stream=None):
        out = self.empty(a.shape[0]) if out is None else out
        check(lib().cy_polysub(self.h, _ptr(a), _ptr(b), _ptr(out), a.shape[0], _stream_handle(stream)),
              "cy_polysub")
        return out

    def scalar_mul(self, a, s: int, out=None, stream=None):
        out = self.empty(a.shape[0]) if out is None else out
        check(lib().cy_poly_scalar_mul(self.h, _ptr(a), limbs_of(s, self.L), _ptr(out), a.shape[0],
                                       _stream_handle(stream)), "cy_poly_scalar_mul")
        return out

    def autotune(self, batch: int = 256, stream=None) -> None:
        check(lib().cy_ring_autotune(self.h, batch, _stream_handle(stream)), "cy_ring_autotune")

    def polymul_graph(self, a, b, out) -> Graph:
        h = ctypes.c_void_p()
        check(lib().cy_polymul_graph_create(self.h, _ptr(a), _ptr(b), _ptr(out), a.shape[0], ctypes.byref(h)),
              "cy_polymul_graph_create")
        return Graph(h, (a, b, out))

    def residues_empty(self, batch: int):
        import torch
        return torch.empty((batch, self.k, self.n), dtype=torch.int32, device="cuda")

    def crt(self, x, out=None, stream=None):
        out = self.residues_empty(x.shape[0]) if out is None else out
        check(lib().cy_crt(self.h, _ptr(x), _ptr(out), x.shape[0], _stream_handle(stream)), "cy_crt")
        return out

    def icrt(self, res, out=None, stream=None):
        out = self.empty(res.shape[0]) if out is None else out
        check(lib().cy_icrt(self.h, _ptr(res), _ptr(out), res.shape[0], _stream_handle(stream)), "cy_icrt")
        return out

    def ntt(self, res, inverse: bool = False, stream=None):
        check(lib().cy_ntt(self.h, _ptr(res), res.shape[0], 1 if inverse else 0, _stream_handle(stream)), "cy_ntt")
        return res


class MixedBatch:
    """A fixed list of products of mixed rings, submitted as one cy_polymul_batched
    call per run. The job array is built once: for a batch of hundreds of jobs,
    building it in Python costs about as much as the GPU work."""

    def __init__(self, jobs: Sequence[tuple]):
        self._jobs = list(jobs)  # keeps the rings and tensors alive
        self.arr = (PolymulJob * len(self._jobs))()
        for i, (r, a, b, c) in enumerate(self._jobs):
            self.arr[i].ring = r.h.value
            self.arr[i].d_a = _ptr(a)
            self.arr[i].d_b = _ptr(b)
            self.arr[i].d_c = _ptr(c)

    def __len__(self) -> int:
        return len(self._jobs)

    def run(self, stream=None) -> None:
        check(lib().cy_polymul_batched(self.arr, len(self._jobs), _stream_handle(stream)), "cy_polymul_batched")


class MixedPlan:
    """A prepared mixed batch (``cy_mixed_plan_*``): polynomial products and YASHE
    multiplies of rings of different N and q, launched as one persistent kernel.

    jobs: ("mul", ring, a, b, c) or ("yashe", scheme, c1, c2, out, relin) with
    device tensors [N][L]. Creation allocates and uploads; ``launch`` issues one
    memset and one kernel, without allocation or host synchronisation."""

    def __init__(self, jobs: Sequence[tuple]):
        self._jobs = list(jobs)
        arr = (MixedJobC * len(self._jobs))()
        for i, j in enumerate(self._jobs):
            if j[0] == "mul":
                _, r, a, b, c = j
                arr[i].ring, arr[i].yashe, arr[i].relin = r.h.value, None, 0
            else:
                _, y, a, b, c, relin = j
                arr[i].ring, arr[i].yashe, arr[i].relin = None, y.h.value, 1 if relin else 0
            arr[i].d_a, arr[i].d_b, arr[i].d_c = _ptr(a), _ptr(b), _ptr(c)
        h = ctypes.c_void_p()
        check(lib().cy_mixed_plan_create(arr, len(self._jobs), ctypes.byref(h)), "cy_mixed_plan_create")
        self.h = h

    def __len__(self) -> int:
        return len(self._jobs)

    def launch(self, stream=None) -> None:
        check(lib().cy_mixed_plan_launch(self.h, _stream_handle(stream)), "cy_mixed_plan_launch")

    def status(self, stream=None) -> None:
        """Raise if a block of the last launch gave up waiting (synchronises)."""
        check(lib().cy_mixed_plan_status(self.h, _stream_handle(stream)), "cy_mixed_plan_status")

    def status_code(self, stream=None) -> int:
        return lib().cy_mixed_plan_status(self.h, _stream_handle(stream))

    @property
    def schedule(self) -> int:
        v = ctypes.c_int(0)
        check(lib().cy_mixed_plan_get_schedule(self.h, ctypes.byref(v)), "cy_mixed_plan_get_schedule")
        return v.value

    @schedule.setter
    def schedule(self, s: int) -> None:
        check(lib().cy_mixed_plan_set_schedule(self.h, s), "cy_mixed_plan_set_schedule")

    def autotune(self, stream=None) -> int:
        check(lib().cy_mixed_plan_autotune(self.h, _stream_handle(stream)), "cy_mixed_plan_autotune")
        return self.schedule

    def graph(self) -> "Graph":
        g = ctypes.c_void_p()
        check(lib().cy_mixed_plan_graph_create(self.h, ctypes.byref(g)), "cy_mixed_plan_graph_create")
        return Graph(g, self)

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().cy_mixed_plan_destroy(self.h)
            self.h = ctypes.c_void_p()


def polymul_batched(jobs: Sequence[tuple], stream=None) -> None:
    """jobs: (ring, a, b, c) with device tensors; one submission for mixed rings."""
    MixedBatch(jobs).run(stream)


def polymul_batched_status(stream=None) -> None:
    """Raise if a block of the last mixed launch gave up waiting (synchronises)."""
    check(lib().cy_polymul_batched_status(_stream_handle(stream)), "cy_polymul_batched_status")


class Yashe:
    """YASHE over Z_q[x]/(x^N+1) on the GPU (handle to a ``cy_yashe``)."""

    def __init__(self, n: int, q: int, t: int, w_bits: int = 32, sigma: float = 8.0):
        self.n, self.q, self.t, self.w_bits, self.sigma = n, q, t, w_bits, sigma
        self.L = nlimbs(q)
        self._qarr = limbs_of(q, self.L)
        p = YasheParams(n=n, q=ctypes.cast(self._qarr, ctypes.POINTER(ctypes.c_uint64)), q_limbs=self.L, t=t,
                        w_bits=w_bits, sigma=sigma)
        h = ctypes.c_void_p()
        check(lib().cy_yashe_create(ctypes.byref(p), ctypes.byref(h)), "cy_yashe_create")
        self.h = h
        rh = ctypes.c_void_p()
        check(lib().cy_yashe_get_ring(h, ctypes.byref(rh)), "cy_yashe_get_ring")
        self.ring = Ring(n, q, handle=rh, owner=self)

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().cy_yashe_destroy(self.h)
            self.h = ctypes.c_void_p()

    def info(self) -> YasheInfo:
        i = YasheInfo()
        check(lib().cy_yashe_get_info(self.h, ctypes.byref(i)), "cy_yashe_get_info")
        return i

    @property
    def ell(self) -> int:
        return self.info().ell

    def autotune(self, batch: int = 256, stream=None) -> None:
        check(lib().cy_yashe_autotune(self.h, batch, _stream_handle(stream)), "cy_yashe_autotune")

    def keygen(self, seed: int) -> None:
        check(lib().cy_yashe_keygen(self.h, seed), "cy_yashe_keygen")

    def set_keys(self, f, h, evk) -> None:
        F = to_limb_array(f, self.L) if not isinstance(f, np.ndarray) else np.ascontiguousarray(f, np.uint64)
        H = to_limb_array(h, self.L) if not isinstance(h, np.ndarray) else np.ascontiguousarray(h, np.uint64)
        EV = to_limb_array(evk, self.L) if not isinstance(evk, np.ndarray) else np.ascontiguousarray(evk, np.uint64)
        check(lib().cy_yashe_set_keys(self.h, F.ctypes.data, H.ctypes.data, EV.ctypes.data), "cy_yashe_set_keys")

    def save_keys(self) -> bytes:
        """The installed keys as one blob (cy_yashe_save_keys)."""
        need = ctypes.c_size_t(0)
        check(lib().cy_yashe_save_keys(self.h, None, 0, ctypes.byref(need)), "cy_yashe_save_keys")
        buf = ctypes.create_string_buffer(need.value)
        check(lib().cy_yashe_save_keys(self.h, buf, need.value, ctypes.byref(need)), "cy_yashe_save_keys")
        return buf.raw

    def load_keys(self, blob: bytes) -> None:
        check(lib().cy_yashe_load_keys(self.h, blob, len(blob)), "cy_yashe_load_keys")

    def get_keys(self):
        F = np.zeros((self.n, self.L), np.uint64)
        H = np.zeros((self.n, self.L), np.uint64)
        EV = np.zeros((self.ell, self.n, self.L), np.uint64)
        check(lib().cy_yashe_get_keys(self.h, F.ctypes.data, H.ctypes.data, EV.ctypes.data), "cy_yashe_get_keys")
        return F, H, EV

    def encrypt_host(self, m: np.ndarray, seed: int) -> np.ndarray:
        m = np.ascontiguousarray(m, dtype=np.uint64)
        if m.ndim == 1:
            m = m[None]
        ct = np.zeros((m.shape[0], self.n, self.L), np.uint64)
        check(lib().cy_yashe_encrypt_host(self.h, m.ctypes.data, ct.ctypes.data, m.shape[0], seed),
              "cy_yashe_encrypt_host")
        return ct

    def encrypt(self, m, seed: int, out=None, stream=None):
        """GPU encryption of device plaintexts m ([batch][N] uint64 words, a CUDA
        tensor) with s and e sampled on the GPU (counter-based, seeded)."""
        out = self.ring.empty(m.shape[0]) if out is None else out
        check(lib().cy_yashe_encrypt(self.h, _ptr(m), _ptr(out), m.shape[0], seed, _stream_handle(stream)),
              "cy_yashe_encrypt")
        return out

    def decrypt(self, ct, aftermul: bool = False, stream=None):
        import torch
        out = torch.empty((ct.shape[0], self.n), dtype=torch.int64, device=ct.device)
        check(lib().cy_yashe_decrypt(self.h, _ptr(ct), _ptr(out), ct.shape[0], 1 if aftermul else 0,
                                     _stream_handle(stream)), "cy_yashe_decrypt")
        return out

    def mul(self, c1, c2, relin: bool = True, out=None, stream=None, workspace: Optional[Workspace] = None):
        out = self.ring.empty(c1.shape[0]) if out is None else out
        st = _stream_handle(stream)
        if workspace is None:
            check(lib().cy_yashe_mul(self.h, _ptr(c1), _ptr(c2), _ptr(out), c1.shape[0], 1 if relin else 0, st),
                  "cy_yashe_mul")
        else:
            check(lib().cy_yashe_mul_ws(self.h, workspace.h, _ptr(c1), _ptr(c2), _ptr(out), c1.shape[0],
                                        1 if relin else 0, st), "cy_yashe_mul_ws")
        return out

    def mul_host(self, c1, c2, out=None, relin: bool = True):
        """The HE multiply on host buffers (numpy arrays or CPU torch tensors,
        [batch][N][L] words); returns once `out` is written."""
        if isinstance(c1, np.ndarray):
            c1 = np.ascontiguousarray(c1, dtype=np.uint64)
            c2 = np.ascontiguousarray(c2, dtype=np.uint64)
        out = (np.empty_like(c1) if isinstance(c1, np.ndarray) else c1.new_empty(c1.shape)) if out is None else out
        check(lib().cy_yashe_mul_host(self.h, _host_ptr(c1), _host_ptr(c2), _host_ptr(out), c1.shape[0],
                                      1 if relin else 0), "cy_yashe_mul_host")
        return out

    def mul_graph(self, c1, c2, out, relin: bool = True) -> Graph:
        h = ctypes.c_void_p()
        check(lib().cy_yashe_mul_graph_create(self.h, _ptr(c1), _ptr(c2), _ptr(out), c1.shape[0], 1 if relin else 0,
                                              ctypes.byref(h)), "cy_yashe_mul_graph_create")
        return Graph(h, (c1, c2, out, self))

    def add_plain(self, c, m, out=None, stream=None):
        """[c + Delta*(m mod t)]_q; m: [batch][N] device words."""
        out = self.ring.empty(c.shape[0]) if out is None else out
        check(lib().cy_yashe_add_plain(self.h, _ptr(c), _ptr(m), _ptr(out), c.shape[0], _stream_handle(stream)),
              "cy_yashe_add_plain")
        return out

    def mul_plain(self, c, m, out=None, stream=None):
        """[c * m_c]_q, m_c the centred representative of m mod t."""
        out = self.ring.empty(c.shape[0]) if out is None else out
        check(lib().cy_yashe_mul_plain(self.h, _ptr(c), _ptr(m), _ptr(out), c.shape[0], _stream_handle(stream)),
              "cy_yashe_mul_plain")
        return out

    def keyswitch(self, c, out=None, stream=None):
        out = self.ring.empty(c.shape[0]) if out is None else out
        check(lib().cy_yashe_keyswitch(self.h, _ptr(c), _ptr(out), c.shape[0], _stream_handle(stream)),
              "cy_yashe_keyswitch")
        return out

    def add(self, c1, c2, out=None, stream=None):
        out = self.ring.empty(c1.shape[0]) if out is None else out
        check(lib().cy_yashe_add(self.h, _ptr(c1), _ptr(c2), _ptr(out), c1.shape[0], _stream_handle(stream)),
              "cy_yashe_add")
        return out


class Server:
    """Continuous-batching request loop (``cy_server``) for YASHE multiplies.

    Requests carry host numpy arrays [N][L] (uint64); the server keeps references
    to them until ``wait`` returns for the ticket.
    """

    def __init__(self, budget_bytes: int, streams: int = 4, max_batch: int = 256, poll_us: int = 20,
                 batch_budget_us: int = 0):
        cfg = ServerConfig(device_budget_bytes=budget_bytes, streams=streams, max_batch=max_batch, poll_us=poll_us,
                           batch_budget_us=batch_budget_us)
        h = ctypes.c_void_p()
        check(lib().cy_server_create(ctypes.byref(cfg), ctypes.byref(h)), "cy_server_create")
        self.h = h
        self._keep = {}
        self._contexts = []

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().cy_server_destroy(self.h)
            self.h = ctypes.c_void_p()
        if getattr(self, "_keep", None):
            self._keep.clear()

    def __del__(self):
        self.close()

    def register(self, y: "Yashe") -> int:
        cid = ctypes.c_int(0)
        check(lib().cy_server_register(self.h, y.h, ctypes.byref(cid)), "cy_server_register")
        self._contexts.append(y)
        return cid.value

    def submit(self, class_id: int, c1: np.ndarray, c2: np.ndarray, out: np.ndarray, relin: bool = True) -> int:
        req = ServeRequest(class_id=class_id, relin=1 if relin else 0, h_c1=c1.ctypes.data, h_c2=c2.ctypes.data,
                           h_out=out.ctypes.data)
        t = ctypes.c_uint64(0)
        check(lib().cy_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)), "cy_server_submit")
        self._keep[t.value] = (c1, c2, out)
        return t.value

    def submit_status(self, class_id: int, c1, c2, out, relin: bool = True) -> int:
        """cy_server_submit's raw status (for rejection tests)."""
        req = ServeRequest(class_id=class_id, relin=1 if relin else 0, h_c1=c1.ctypes.data if c1 is not None else 0,
                           h_c2=c2.ctypes.data if c2 is not None else 0, h_out=out.ctypes.data if out is not None else 0)
        t = ctypes.c_uint64(0)
        return lib().cy_server_submit(self.h, ctypes.byref(req), ctypes.byref(t))

    def submit_device(self, class_id, c1, c2, out, relin=True) -> list:
        """Queues requests on device-resident ciphertexts (``cy_server_submit_device``).

        c1, c2, out: int64 CUDA tensors [count][N][L] (one request per row) or
        sequences of device addresses; ``relin`` and ``class_id`` apply to every
        request, or are per-request sequences. Returns the tickets."""
        def addrs(x):
            if hasattr(x, "data_ptr"):
                step = x.stride(0) * x.element_size() if x.dim() == 3 else 0  # 0 for an expanded tensor
                return [x.data_ptr() + i * step for i in range(x.shape[0] if x.dim() == 3 else 1)]
            return [int(a) for a in x]
        a1, a2, ao = addrs(c1), addrs(c2), addrs(out)
        n = len(a1)
        cls = class_id if hasattr(class_id, "__len__") else [class_id] * n
        rl = relin if hasattr(relin, "__len__") else [relin] * n
        reqs = (ServeRequestDev * n)()
        for i in range(n):
            reqs[i].class_id = int(cls[i])
            reqs[i].relin = 1 if rl[i] else 0
            reqs[i].d_c1, reqs[i].d_c2, reqs[i].d_out = a1[i], a2[i], ao[i]
        t = (ctypes.c_uint64 * n)()
        check(lib().cy_server_submit_device(self.h, reqs, n, t), "cy_server_submit_device")
        return list(t)

    def submit_device_raw(self, reqs, n: int, tickets) -> int:
        """``cy_server_submit_device`` on prepared ctypes arrays (no conversion)."""
        return lib().cy_server_submit_device(self.h, reqs, n, tickets)

    def poll(self, ticket: int) -> bool:
        d = ctypes.c_int(0)
        check(lib().cy_server_poll(self.h, ticket, ctypes.byref(d)), "cy_server_poll")
        return bool(d.value)

    def wait(self, ticket: int, timeout_ms: int = 60000) -> None:
        st = lib().cy_server_wait(self.h, ticket, timeout_ms)
        if st != -7:  # still queued on a timeout: keep its buffers alive
            self._keep.pop(ticket, None)
        check(st, "cy_server_wait")

    def drain(self, timeout_ms: int = 600000) -> None:
        check(lib().cy_server_drain(self.h, timeout_ms), "cy_server_drain")

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(lib().cy_server_get_stats(self.h, ctypes.byref(s)), "cy_server_get_stats")
        return s

    def reset_stats(self) -> None:
        check(lib().cy_server_reset_stats(self.h), "cy_server_reset_stats")


__all__ = ["Server", "Ring", "Yashe", "Workspace", "Graph", "MixedPlan", "polymul_batched", "polymul_batched_status", "to_limb_array", "from_limb_array", "to_device",
           "to_host", "nlimbs", "CY_OK"]
