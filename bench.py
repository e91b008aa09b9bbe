#!/usr/bin/env python3
"""Benchmark of the cuYASHE hot path on GB300.

Workload (one step): one batched YASHE homomorphic multiply with
relinearisation, N = 4096, q = a 127-bit prime (q = 1 mod 2^16), t = 1024,
w = 2^32 (4 digits), over B ciphertext pairs resident in HBM
(cy_yashe_mul, relin = 1). Reported beside it, outside the headline:
  * the plain per-call path (one HE multiply per call, synchronised),
  * batched and per-call polynomial products at N = 4096, q = 2^127 - 1,
  * e2e: the same multiply through host buffers with the copies timed,
  * per-kernel device times (CUDA events) and the roofline of the top kernel,
  * the reference's CPU multiply (C restatement) timed on the host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "polymul/s & HE mults/s at N=4096, batched vs plain, bit-exact; % HBM roofline"
N = 4096
Q_YASHE = 170141183460469231731687303715883253761  # largest prime < 2^127 with q = 1 (mod 2^16)
Q_POLY = 2**127 - 1                                 # the reference benchmark's q
T = 1024
W_BITS = 32
L = 2                                               # uint64 limbs per coefficient
CT_BYTES = N * L * 8                                # one ciphertext / polynomial
DEEP_N, DEEP_T, DEEP_PAIRS = 16384, 65537, 64       # the deep-level workload


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.skip = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()  # start timing only once the sampler is producing
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = len(self.lines)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[max(0, self.skip - 1):]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# reference arm / CPU baseline: the oracle's C restatement of the reference
# ----------------------------------------------------------------------------

def cpu_yashe_rate(pairs: int, threads: int, c1, c2, evk):
    """HE mults/s of the reference's multiply (restated in C) on `pairs` pairs."""
    from oracle import refpath

    rp = refpath.RefPath(Q_YASHE, N)
    t0 = time.perf_counter()
    rp.yashe_mul(c1[:pairs], c2[:pairs], T, W_BITS, evk, nthreads=threads)
    dt = time.perf_counter() - t0
    return pairs / dt, dt


def synthetic_host_cts(pairs: int, seed: int):
    """Ciphertext-shaped inputs uniform in [0, 2^126) (below q; fresh YASHE
    ciphertexts are computationally indistinguishable from uniform) and an
    evaluation key of the same shape (4 digits)."""
    import numpy as np

    rng = np.random.default_rng(seed)

    def uni(shape):
        lo = rng.integers(0, 2**64, size=shape, dtype=np.uint64)
        hi = rng.integers(0, 2**62, size=shape, dtype=np.uint64)
        return np.ascontiguousarray(np.stack([lo, hi], axis=-1))
    return uni((pairs, N)), uni((pairs, N)), uni((4, N))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    c1, c2, evk = synthetic_host_cts(max(threads, 8), 1)
    pairs = max(threads, 8)
    rates = []
    for _ in range(args.warmup):
        cpu_yashe_rate(min(pairs, threads), threads, c1, c2, evk)
    for _ in range(args.steps):
        r, _ = cpu_yashe_rate(pairs, threads, c1, c2, evk)
        rates.append(r)
    v = statistics.median(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "HE mults/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * pairs / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": "yashe_mul_relin N=4096 log2q=127 t=1024 w=2^32 ell=4",
                   "implementation": "the reference's CPU multiply restated in C (oracle/refpath.c)",
                   "pairs_per_step": pairs, "host_threads": threads},
        "cpu_baseline": {"value": v, "unit": "HE mults/s", "cores": threads, "kind": "port",
                         "sample": "%d HE multiplies per step at N=4096 (29-bit CRT bucket, Goldilocks Stockham NTT)"
                                   % pairs},
        "e2e": {"value": v, "unit": "HE mults/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# serving (Poisson arrivals of mixed-size HE multiplies)
# ----------------------------------------------------------------------------

SERVE_CLASSES = [  # (N, q, t, weight): q = largest prime below 2^b with q = 1 (mod 2^16)
    # t = 17 for the 62-bit q: with t = 257 a relinearised product's noise reaches
    # half a plaintext step (rounding distance 0.4999) and decryption fails; with
    # t = 17 the worst distance is 0.009
    (2048, 4611686018427322369, 17, 0.4),
    (4096, Q_YASHE, 1024, 0.3),
    (8192, 1569275433846670190958947355801916604025588861116000698369, 65537, 0.2),
    (16384, None, 65537, 0.1),
]


def _q380():
    # largest prime below 2^380 with q = 1 (mod 2^16); primality by Miller-Rabin
    def is_prime(n):
        d, r = n - 1, 0
        while d % 2 == 0:
            d //= 2
            r += 1
        for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
            x = pow(a, d, n)
            if x in (1, n - 1):
                continue
            for _ in range(r - 1):
                x = x * x % n
                if x == n - 1:
                    break
            else:
                return False
        return True
    p = ((2**380 - 2) >> 16 << 16) + 1
    while not is_prime(p):
        p -= 1 << 16
    return p


SERVE_P99_BOUND_MS = 10.0  # latency bound of the capacity figure
SERVE_SWEEP = (20000.0, 40000.0, 80000.0, 160000.0, 240000.0, 320000.0)  # offered rates of the capacity sweep


def _poisson(rng, rate_per_s, count):
    import numpy as np

    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=count))


def _resident_run(srv, classes, ids, dev, rate_per_s, seconds, seed):
    """Poisson arrivals of requests on device-resident ciphertexts, submitted in
    arrival order (every request due by now in one cy_server_submit_device
    call); returns the server's statistics of the run."""
    import ctypes

    import numpy as np

    from cuyashe_gb300 import ServeRequestDev

    rng = np.random.default_rng(seed)
    count = int(rate_per_s * seconds)
    arrivals = _poisson(rng, rate_per_s, count)
    weights = np.array([c["w"] for c in classes])
    kinds = rng.choice(len(classes), size=count, p=weights / weights.sum())
    picks = rng.integers(0, 8, size=(count, 2))
    # requests prepared up front as one array of cy_serve_request_dev records
    rec = np.zeros(count, dtype=np.dtype([("cls", "<i4"), ("relin", "<i4"), ("c1", "<u8"), ("c2", "<u8"),
                                          ("out", "<u8")]))
    assert rec.dtype.itemsize == ctypes.sizeof(ServeRequestDev)
    base_ct = np.array([dev[k][0].data_ptr() for k in range(len(classes))], np.uint64)
    base_out = np.array([dev[k][1].data_ptr() for k in range(len(classes))], np.uint64)
    poly_b = np.array([c["poly_bytes"] for c in classes], np.uint64)
    slots = np.array([dev[k][1].shape[0] for k in range(len(classes))], np.uint64)
    pool = np.array([c["pool"] for c in classes], np.uint64)
    rec["cls"] = np.array(ids)[kinds]
    rec["relin"] = 1
    rec["c1"] = base_ct[kinds] + picks[:, 0].astype(np.uint64) * poly_b[kinds]
    rec["c2"] = base_ct[kinds] + (pool[kinds] + picks[:, 1].astype(np.uint64)) * poly_b[kinds]
    rec["out"] = base_out[kinds] + (np.arange(count, dtype=np.uint64) % slots[kinds]) * poly_b[kinds]
    tickets = (ctypes.c_uint64 * count)()
    rsz, tsz = rec.dtype.itemsize, ctypes.sizeof(ctypes.c_uint64)
    rbase, tbase = rec.ctypes.data, ctypes.addressof(tickets)
    srv.reset_stats()
    i = 0
    t0 = time.perf_counter()
    while i < count:
        j = int(np.searchsorted(arrivals, time.perf_counter() - t0, side="right"))
        if j > i:
            st = srv.submit_device_raw(ctypes.cast(rbase + i * rsz, ctypes.POINTER(ServeRequestDev)), j - i,
                                       ctypes.cast(tbase + i * tsz, ctypes.POINTER(ctypes.c_uint64)))
            if st != 0:
                raise RuntimeError("cy_server_submit_device: %d" % st)
            i = j
    lag_ms = (time.perf_counter() - t0 - arrivals[-1]) * 1000.0  # submission lag at the end of the trace
    srv.drain()
    for t in tickets:
        srv.wait(t)
    st = srv.stats()
    return {"requests": count, "offered_rate_per_s": rate_per_s, "throughput_per_s": st.throughput_per_s,
            "p50_ms": st.p50_us / 1000.0, "p99_ms": st.p99_us / 1000.0, "mean_ms": st.mean_us / 1000.0,
            "batches": int(st.batches), "mean_batch": count / max(1, int(st.batches)), "failed": int(st.failed),
            "submit_lag_ms": round(lag_ms, 3)}


def serving_bench(cy, rate_per_s=20000.0, seconds=1.0, plain_prefix=2000, seed=2024, batch_budget_us=0,
                  sweep=SERVE_SWEEP, sweep_seconds=1.0):
    import numpy as np
    import torch

    from cuyashe_gb300.api import Ring, Server, Yashe

    classes = []
    for n, q, t, w in SERVE_CLASSES:
        q = q or _q380()
        y = Yashe(n, q, t)
        y.keygen(n + 17)
        pool = 8
        rng = np.random.default_rng(n)
        m = rng.integers(0, t, size=(2 * pool, n), dtype=np.uint64)
        ct = y.encrypt_host(m, seed=n)
        classes.append({"y": y, "w": w, "ct": ct, "m": m, "t": t, "pool": pool, "n": n, "qbits": q.bit_length(),
                        "poly_bytes": ct[0].nbytes})
    rng = np.random.default_rng(seed)
    count = int(rate_per_s * seconds)
    arrivals = _poisson(rng, rate_per_s, count)
    weights = np.array([c["w"] for c in classes])
    kinds = rng.choice(len(classes), size=count, p=weights / weights.sum())
    picks = rng.integers(0, 8, size=(count, 2))
    outs = [np.zeros((256,) + c["ct"].shape[1:], np.uint64) for c in classes]  # reused cyclically

    srv = Server(budget_bytes=120 << 30, streams=4, max_batch=256, batch_budget_us=batch_budget_us)
    ids = [srv.register(c["y"]) for c in classes]
    # warm-up: a burst of every class, so that slots and workspaces have grown to
    # the batch sizes of the run before it is timed
    warm = [srv.submit(ids[k], c["ct"][i % 8], c["ct"][c["pool"] + (i * 3) % 8], outs[k][i])
            for k, c in enumerate(classes) for i in range(64)]
    for t in warm:
        srv.wait(t)
    # the first 8 served products of every class decrypt to m1 * m2 mod t (slot i
    # holds ct[i] * ct[pool + 3i mod 8]; checked before the timed run reuses the slots)
    decrypt_ok = True
    for k, c in enumerate(classes):
        got = c["y"].decrypt(torch.from_numpy(outs[k][0:8].view(np.int64)).cuda()).cpu().numpy().view(np.uint64)
        PT = Ring(c["n"], c["t"])
        exp = PT.polymul(PT.upload([c["m"][i].tolist() for i in range(8)]),
                         PT.upload([c["m"][c["pool"] + (i * 3) % 8].tolist() for i in range(8)]))
        decrypt_ok = decrypt_ok and bool((got == exp.cpu().numpy().view(np.uint64)[..., 0]).all())
    srv.reset_stats()
    tickets = []
    t0 = time.perf_counter()
    for i in range(count):
        while time.perf_counter() - t0 < arrivals[i]:
            pass
        k = int(kinds[i])
        c = classes[k]
        tickets.append(srv.submit(ids[k], c["ct"][picks[i, 0]], c["ct"][c["pool"] + picks[i, 1]],
                                  outs[k][i % 256]))
    srv.drain()
    for t in tickets:
        srv.wait(t)
    st = srv.stats()
    served = {"requests": count, "offered_rate_per_s": rate_per_s, "throughput_per_s": st.throughput_per_s,
              "p50_ms": st.p50_us / 1000.0, "p99_ms": st.p99_us / 1000.0, "mean_ms": st.mean_us / 1000.0,
              "batches": int(st.batches), "mean_batch": count / max(1, int(st.batches)), "failed": int(st.failed),
              "peak_device_gb": st.peak_device_bytes / 1e9, "batch_budget_us": batch_budget_us,
              "api": "cy_server_submit (host buffers, copied in and out per request)",
              "mix": {"%d/%d/t=%d" % (c["n"], c["qbits"], c["t"]): c["w"] for c in classes}}

    srv.close()

    # ciphertexts resident in HBM: uploaded once, results left on the device. A
    # server with more slots and larger batches (no host staging to grow), warmed
    # with a burst of full batches of every class so that slots have their size.
    srv = Server(budget_bytes=120 << 30, streams=8, max_batch=512, batch_budget_us=batch_budget_us)
    ids = [srv.register(c["y"]) for c in classes]
    dev = {}
    for k, c in enumerate(classes):
        dev[k] = (torch.from_numpy(c["ct"].view(np.int64)).cuda(),
                  torch.zeros((2048,) + c["ct"].shape[1:], dtype=torch.int64, device="cuda"))
    torch.cuda.synchronize()
    for k in range(len(classes)):  # 8 full batches per class: every slot grows to every class's size
        d_ct, d_out = dev[k]
        burst = []
        for _ in range(8):
            burst += srv.submit_device(ids[k], d_ct[:1].expand(512, -1, -1), d_ct[8:9].expand(512, -1, -1),
                                       d_out[:512])
        for t in burst:
            srv.wait(t)
    _resident_run(srv, classes, ids, dev, 20000.0, 0.25, seed + 1)  # warm-up of the device path
    resident = _resident_run(srv, classes, ids, dev, rate_per_s, seconds, seed + 2)
    resident["api"] = "cy_server_submit_device (ciphertexts and results in device memory)"
    # capacity: offered rates until the server no longer keeps up within the bound
    points = []
    capacity = 0.0
    for r in sweep:
        pt = _resident_run(srv, classes, ids, dev, r, sweep_seconds, seed + int(r))
        points.append({k: pt[k] for k in ("offered_rate_per_s", "throughput_per_s", "p50_ms", "p99_ms",
                                           "mean_batch", "submit_lag_ms")})
        ok = pt["throughput_per_s"] >= 0.95 * r and pt["p99_ms"] <= SERVE_P99_BOUND_MS and pt["failed"] == 0
        if ok:
            capacity = r
        else:
            break
    srv.close()
    del dev

    # the plain per-request path on the same trace prefix: one multiply per
    # request, in arrival order, host buffers copied in and out each time
    lat = []
    devp = {}
    for k, c in enumerate(classes):
        shp = c["ct"].shape[1:]
        devp[k] = (torch.empty((1,) + shp, dtype=torch.int64, device="cuda"),
                   torch.empty((1,) + shp, dtype=torch.int64, device="cuda"),
                   torch.empty((1,) + shp, dtype=torch.int64, device="cuda"))
    pinned = {k: torch.from_numpy(c["ct"].view(np.int64)).pin_memory() for k, c in enumerate(classes)}
    t0 = time.perf_counter()
    for i in range(min(plain_prefix, count)):
        while time.perf_counter() - t0 < arrivals[i]:
            pass
        k = int(kinds[i])
        c = classes[k]
        d1, d2, do = devp[k]
        d1[0].copy_(pinned[k][picks[i, 0]], non_blocking=True)
        d2[0].copy_(pinned[k][c["pool"] + picks[i, 1]], non_blocking=True)
        c["y"].mul(d1, d2, relin=True, out=do)
        do.cpu()
        lat.append(time.perf_counter() - t0 - arrivals[i])
    span = time.perf_counter() - t0
    lat = np.array(lat) * 1000.0
    plain = {"requests": len(lat), "throughput_per_s": len(lat) / span, "p50_ms": float(np.percentile(lat, 50)),
             "p99_ms": float(np.percentile(lat, 99))}
    out = {"continuous_batching": served, "resident": resident,
           "capacity": {"p99_bound_ms": SERVE_P99_BOUND_MS, "capacity_per_s": capacity, "sweep": points,
                        "api": "cy_server_submit_device", "seconds_per_rate": sweep_seconds},
           "plain_per_request": plain, "decrypt_ok": decrypt_ok, "decrypt_checked_per_class": 8}
    if not decrypt_ok:  # a wrong product invalidates every serving figure
        out = {"invalid": "decryption of served products failed", "decrypt_ok": False}
    return out


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------

def make_inputs(Y, batch: int, pool: int, seed: int, n: int = N, t: int = T):
    """Fresh encryptions (library keygen + encryption), tiled to `batch` pairs."""
    import numpy as np
    import torch

    rng = np.random.default_rng(seed)
    m1 = rng.integers(0, t, size=(pool, n), dtype=np.uint64)
    m2 = rng.integers(0, t, size=(pool, n), dtype=np.uint64)
    ct1 = Y.encrypt_host(m1, seed=seed + 1)
    ct2 = Y.encrypt_host(m2, seed=seed + 2)
    idx1 = np.arange(batch) % pool
    idx2 = (np.arange(batch) * 7 + 3) % pool
    C1 = torch.from_numpy(ct1.view(np.int64)).cuda()[torch.from_numpy(idx1).cuda()].contiguous()
    C2 = torch.from_numpy(ct2.view(np.int64)).cuda()[torch.from_numpy(idx2).cuda()].contiguous()
    return C1, C2, m1, m2, idx1, idx2


def deep_bench(cy, steps: int, stream):
    """The deep-level workload: 64 HE multiplies with relinearisation at
    N = 16384, a 380-bit q (the largest prime below 2^380 that is 1 mod 2^16),
    t = 65537, w = 2^32 (12 digits). Its inputs (100 MB) fit in L2, so every
    step is timed alone with CUDA events after a write of a buffer larger than
    L2, and the step times are summed."""
    import numpy as np
    import torch

    q = _q380()
    Y = cy.Yashe(DEEP_N, q, DEEP_T, W_BITS, 8.0)
    Y.keygen(4242)
    Y.autotune(batch=DEEP_PAIRS)
    C1, C2, m1, m2, i1, i2 = make_inputs(Y, DEEP_PAIRS, pool=4, seed=31, n=DEEP_N, t=DEEP_T)
    OUT = Y.ring.empty(DEEP_PAIRS)

    def step():
        Y.mul(C1, C2, relin=True, out=OUT)

    step()
    dec = Y.decrypt(OUT[:2]).cpu().numpy().view(np.uint64)
    PT = cy.Ring(DEEP_N, DEEP_T)
    exp = PT.polymul(PT.upload(m1[i1[:2]].astype(object).tolist()),
                     PT.upload(m2[i2[:2]].astype(object).tolist()))
    exp = exp.cpu().numpy().view(np.uint64)[..., 0]
    ok = bool((dec == exp).all())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        step()
    total = 0.0
    for _ in range(steps):
        flush.fill_(1)
        total += time_steps(step, 1, stream)
    cy.lib().cy_set_chunk_overlap(0)  # serial chunks: each kernel's own event times
    with cy.Trace() as tr:
        step()
    cy.lib().cy_set_chunk_overlap(1)
    kernels = {name: {"launches": cnt, "ms": round(kms, 4)} for name, (cnt, kms) in tr.kernels.items()}
    info = Y.info()
    return {"workload": "yashe_mul_relin N=16384 log2q=%d t=%d w=2^32 ell=%d" % (q.bit_length(), DEEP_T, info.ell),
            "pairs": DEEP_PAIRS, "he_mults_per_s": DEEP_PAIRS * steps / (total / 1000.0),
            "ms_per_step": total / steps, "tensor_primes": info.tensor_primes, "relin_primes": info.relin_primes,
            "l2": "256 MB written between timed steps", "kernels": kernels, "decrypt_check": ok,
            "schedules": ";".join(x for x in cy.tuning_export().split(";") if x.startswith("n16384"))}


def ncu_deep_step(pairs: int):
    """One autotuned deep-level HE multiply of `pairs` pairs between
    cudaProfilerStart/Stop (for ncu --profile-from-start off)."""
    import numpy as np
    import torch

    import cuyashe_gb300 as cy

    Y = cy.Yashe(DEEP_N, _q380(), DEEP_T, W_BITS, 8.0)
    Y.keygen(4242)
    Y.autotune(batch=pairs)
    C1, C2, _, _, _, _ = make_inputs(Y, pairs, pool=4, seed=31, n=DEEP_N, t=DEEP_T)
    out = Y.ring.empty(pairs)
    for _ in range(3):
        Y.mul(C1, C2, relin=True, out=out)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    Y.mul(C1, C2, relin=True, out=out)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    log("ncu deep step done:", ";".join(x for x in cy.tuning_export().split(";") if x.startswith("n16384")))


def time_steps(fn, steps: int, stream):
    import torch

    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(steps):
        fn()
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end)


def kernel_counts(tuning: str) -> dict:
    """Warp instructions and DRAM bytes per job of the kernels of the headline
    step, for the schedules in `tuning` (cy_tuning_export), from the committed ncu
    summary profiles/kernel_counts_n4096.json; {} when it has no such entry."""
    path = os.path.join(ROOT, "profiles", "kernel_counts_n4096.json")
    if not os.path.exists(path):
        return {}
    per = json.load(open(path))["per_unit"]
    tuned = dict(item.split("=") for item in tuning.split(";") if item.startswith("n4096.l2."))
    out = {}
    for name, op in (("mul_centered", "mulc"), ("keyswitch", "ks"), ("mul", "mul")):
        key = "%s=%s" % (op, tuned.get("n4096.l2." + op, "0"))
        if key in per:
            out[name] = dict(per[key], source=key)
    for name in ("epi_yashe", "epi_modq"):
        if name in per:
            out[name] = dict(per[name], source=name)
    return out


def int_roofline(kernels: dict, counts: dict, jobs: int, sm_mhz: float, sms: int, ms_per_step: float):
    """Issue-slot roofline of the integer-bound kernels: executed warp
    instructions (ncu, per job) x jobs / kernel time, against SMs x 4 schedulers
    x the sampled SM clock. One row per kernel of the step and the whole step."""
    if not counts or not sm_mhz:
        return None
    peak = sms * 4 * sm_mhz * 1e6  # warp instructions per second
    rows = {}
    step_inst = 0.0
    for name, k in kernels.items():
        c = counts.get(name.split("_n")[0])
        if not c or k["ms"] <= 0:
            continue
        inst = c["warp_inst"] * jobs
        step_inst += inst
        rate = inst / (k["ms"] / 1000.0)
        rows[name] = {"warp_inst_per_launch": inst / k["launches"], "achieved": rate, "frac": round(rate / peak, 4),
                      "schedule": c["source"]}
    top = max(kernels, key=lambda n: kernels[n]["ms"])
    return {"bound": "issue", "unit": "warp instructions/s", "peak": peak,
            "peak_basis": "%d SMs x 4 schedulers x %.0f MHz (median sampled SM clock)" % (sms, sm_mhz),
            "kernel": top, "achieved": rows.get(top, {}).get("achieved"), "frac": rows.get(top, {}).get("frac"),
            "kernels": rows, "step_frac": round(step_inst / (ms_per_step / 1000.0) / peak, 4),
            "source": "profiles/kernel_counts_n4096.json (ncu smsp__inst_executed.sum per job)"}


def kernel_bytes(name: str, launches: int, jobs: int, k_tensor: int, k_relin: int, ell: int):
    """Algorithmic bytes moved by all launches of one kernel over `jobs` jobs."""
    res = N * 4
    if name.startswith("mul_centered"):
        return jobs * (2 * CT_BYTES + k_tensor * res)
    if name.startswith("keyswitch"):
        return jobs * (CT_BYTES + k_relin * res) + launches * ell * k_relin * N * 8
    if name.startswith("epi_yashe"):
        return jobs * (k_tensor * res + CT_BYTES)
    if name.startswith("epi_modq"):
        return jobs * (k_relin * res + CT_BYTES)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import cuyashe_gb300 as cy

    from cuyashe_gb300 import replicas

    rep = replicas.from_env("nccl")  # replicas: no data-path collective
    world, rank, local = rep.world, rep.rank, rep.local
    cy.lib()
    stream = torch.cuda.current_stream()
    B = args.batch

    # ---- set-up (untimed): keys, schedule autotuning, fresh encryptions --------
    Y = cy.Yashe(N, Q_YASHE, T, W_BITS, 8.0)
    Y.keygen(1234 + rank)
    if args.schedules:  # pinned (a profiled run: timings under ncu would mislead the tuner)
        cy.tuning_import(args.schedules)
    elif not args.no_autotune:
        Y.autotune(batch=B)  # the schedules that are fastest at the step's own batch
    tuning = cy.tuning_export()
    # weak scaling: each rank multiplies its own contiguous share (B pairs) of the
    # job's world * B pairs; no data-path collective
    p_start, p_stop = replicas.shard(world * B, rank, world)
    C1, C2, m1, m2, idx1, idx2 = make_inputs(Y, p_stop - p_start, pool=32, seed=77 + p_start)
    OUT = Y.ring.empty(B)
    Y.mul(C1, C2, relin=True, out=OUT)
    dec = Y.decrypt(OUT[:4]).cpu().numpy().view(np.uint64)
    PT = cy.Ring(N, T)  # plaintext ring Z_t[x]/(x^N+1): reference products on the GPU
    exp = PT.polymul(PT.upload(m1[idx1[:4]].astype(object).tolist()),
                     PT.upload(m2[idx2[:4]].astype(object).tolist()))
    exp = exp.cpu().numpy().view(np.uint64)[..., 0]
    torch.cuda.synchronize()
    decrypt_ok = bool((dec == exp).all())
    log("decrypt(c1*c2) == m1*m2 mod t:", decrypt_ok)

    def step():
        Y.mul(C1, C2, relin=True, out=OUT)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if args.ncu_step:
        # one step between cudaProfilerStart/Stop for `ncu --profile-from-start off`
        torch.cuda.profiler.start()
        step()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        log("ncu step done")
        return

    # ---- timed region -----------------------------------------------------------
    launches0 = cy.launch_count()
    replicas.barrier(rep)
    with ClockSampler(local) as clocks:
        ms = time_steps(step, args.steps, stream)
    launches = cy.launch_count() - launches0
    ms_max = replicas.max_over_ranks(rep, ms)
    value = world * B * args.steps / (ms_max / 1000.0)
    log("batched HE mults/s: %.1f (%.3f ms/step, batch %d)" % (value, ms_max / args.steps, B))

    if rank != 0:
        replicas.close(rep)
        return

    # ---- per-kernel device times (one traced step, outside the timed region) ----
    # The timed steps overlap the kernels of neighbouring chunks on two streams;
    # this step runs its chunks one after another so that each kernel's event
    # times are its own (the roofline's per-launch durations and the shares).
    info = Y.info()
    cy.lib().cy_set_chunk_overlap(0)
    with cy.Trace() as tr:
        step()
    cy.lib().cy_set_chunk_overlap(1)
    kernels = {}
    for name, (cnt, kms) in tr.kernels.items():
        kernels[name] = {"launches": cnt, "ms": round(kms, 4)}
    total_k = sum(v["ms"] for v in kernels.values()) or 1.0
    for v in kernels.values():
        v["share"] = round(v["ms"] / total_k, 4)
    top = max(kernels, key=lambda k: kernels[k]["ms"])
    peak, peak_kind = read_peaks()
    top_bytes = kernel_bytes(top, kernels[top]["launches"], B, info.tensor_primes, info.relin_primes, info.ell)
    top_gbs = top_bytes / (kernels[top]["ms"] / 1000.0) / 1e9
    # measured counts per job of the schedule each kernel ran with (ncu, committed summary)
    counts = kernel_counts(tuning)
    traffic = None
    top_counts = counts.get(top.split("_n")[0])
    if top_counts:
        traffic = top_counts["dram_bytes"] * B / kernels[top]["launches"]
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(top_gbs, 1), "peak": peak, "unit": "GB/s",
                "frac": round(top_gbs / peak, 4), "peak_kind": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": top_bytes / kernels[top]["launches"],
                "traffic_source": top_counts["source"] if top_counts else None}
    step_bytes = B * 3 * CT_BYTES + info.ell * N * L * 8
    step_gbs = step_bytes / (ms_max / args.steps / 1000.0) / 1e9

    # ---- e2e: host buffers through cy_yashe_mul_host, copies inside the timed region
    # (measured right after the device-buffer steps, before the other sections)
    # (the call pipelines chunks: copies of one chunk overlap the kernels of the next)
    H1 = C1.cpu().pin_memory()
    H2 = C2.cpu().pin_memory()
    HO = torch.empty_like(H1).pin_memory()

    def e2e_step():
        Y.mul_host(H1, H2, out=HO, relin=True)

    e2e_step()
    # four windows of calls, the median window reported: host-memory traffic from
    # other tenants of the machine stalls the copies now and then, and one stall
    # should not set the figure (every window's rate is in the line)
    e2e_per_window = max(3, args.steps // 2)
    e2e_windows = []
    torch.cuda.synchronize()
    for _ in range(4):
        t0 = time.perf_counter()
        for _ in range(e2e_per_window):
            e2e_step()
        e2e_windows.append(B * e2e_per_window / (time.perf_counter() - t0))
    e2e_rate = statistics.median(e2e_windows)
    e2e_ok = torch.equal(HO, OUT.cpu())
    # copy bandwidth on its own (what bounds e2e when the copies outlast the kernels)
    Dtmp = torch.empty_like(C1)
    h2d_ms = time_steps(lambda: Dtmp.copy_(H1, non_blocking=True), 5, stream)
    d2h_ms = time_steps(lambda: HO.copy_(OUT, non_blocking=True), 5, stream)
    copy_gbs = {"h2d_gbs": 5 * B * CT_BYTES / (h2d_ms / 1000.0) / 1e9,
                "d2h_gbs": 5 * B * CT_BYTES / (d2h_ms / 1000.0) / 1e9}
    del Dtmp

    # ---- plain per-call path: one HE multiply per call, synchronised ------------
    plain_calls = 200
    o1 = Y.ring.empty(1)

    def plain():
        for j in range(plain_calls):
            Y.mul(C1[j:j + 1], C2[j:j + 1], relin=True, out=o1)
            torch.cuda.synchronize()
    plain()
    t0 = time.perf_counter()
    plain()
    plain_rate = plain_calls / (time.perf_counter() - t0)

    # ---- CUDA graphs: the batched step and a one-pair call, replayed ----------
    graphs = None
    try:
        g_step = Y.mul_graph(C1, C2, OUT, relin=True)
        g_step.launch()
        torch.cuda.synchronize()
        g_ms = time_steps(lambda: g_step.launch(stream), args.steps, stream)
        g_one = Y.mul_graph(C1[:1], C2[:1], o1, relin=True)
        g_one.launch()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in range(plain_calls):
            g_one.launch(stream)
            torch.cuda.synchronize()
        graphs = {"batched_he_mults_per_s": B * args.steps / (g_ms / 1000.0),
                  "per_call_he_mults_per_s": plain_calls / (time.perf_counter() - t0)}
        del g_step, g_one
    except Exception as e:
        log("graph replay failed:", e)

    # ---- polynomial products (Polynomial c = a*b; c.reduce()) ------------------
    R = cy.Ring(N, Q_POLY)
    if not args.no_autotune:
        R.autotune(batch=512)
    PB = B
    rng = np.random.default_rng(5)
    A = torch.from_numpy((rng.integers(0, 2**63, size=(PB, N, L), dtype=np.uint64)).view(np.int64)).cuda()
    Bp = torch.from_numpy((rng.integers(0, 2**63, size=(PB, N, L), dtype=np.uint64)).view(np.int64)).cuda()
    A[..., 1] &= (1 << 62) - 1  # < 2^126 < q
    Bp[..., 1] &= (1 << 62) - 1
    Cp = R.empty(PB)
    R.polymul(A, Bp, out=Cp)
    poly_ms = time_steps(lambda: R.polymul(A, Bp, out=Cp), args.steps, stream)
    poly_rate = PB * args.steps / (poly_ms / 1000.0)
    c1p = R.empty(1)
    t0 = time.perf_counter()
    for j in range(plain_calls):
        R.polymul(A[j:j + 1], Bp[j:j + 1], out=c1p)
        torch.cuda.synchronize()
    poly_plain = plain_calls / (time.perf_counter() - t0)
    # end to end on page-locked host buffers (copies inside, host wall clock)
    HA, HB = A.cpu().pin_memory(), Bp.cpu().pin_memory()
    HC = torch.empty_like(HA).pin_memory()
    R.polymul_host(HA, HB, out=HC)
    e2e_reps = max(3, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_reps):
        R.polymul_host(HA, HB, out=HC)
    poly_e2e = PB * e2e_reps / (time.perf_counter() - t0)
    poly_e2e_ok = torch.equal(HC, Cp.cpu())
    del HA, HB, HC

    # ---- standalone NTT kernel (cy_ntt) against the HBM roofline -----------------
    # One read and one write of every 32-bit residue per transform are the
    # algorithmic bytes; [4096][9][4096] residues (604 MB, above L2).
    ntt_line = None
    try:
        kq = R.k
        RES = torch.zeros((PB, kq, N), dtype=torch.int32, device="cuda")
        R.ntt(RES)
        R.ntt(RES, inverse=True)
        reps = max(10, args.steps)  # ~0.3 ms a call: enough calls for a steady mean
        f_ms = time_steps(lambda: R.ntt(RES), reps, stream)
        i_ms = time_steps(lambda: R.ntt(RES, inverse=True), reps, stream)
        nbytes = 2 * RES.numel() * 4
        fg = nbytes * reps / (f_ms / 1000.0) / 1e9
        ig = nbytes * reps / (i_ms / 1000.0) / 1e9
        ntt_line = {"transforms": PB * kq, "n": N, "forward_gbs": round(fg, 1), "inverse_gbs": round(ig, 1),
                    "peak_gbs": peak, "forward_frac": round(fg / peak, 4), "inverse_frac": round(ig / peak, 4),
                    "transforms_per_s": PB * kq * reps / (f_ms / 1000.0),
                    "schedule": ";".join(x for x in cy.tuning_export().split(";") if ".ntt=" in x)}
        log("standalone NTT:", ntt_line)
        del RES
    except Exception as e:
        log("ntt bench failed:", e)

    # ---- mixed batch: 512 products, N over {1024..8192}, q of 62/127/190 bits, ---
    # ---- and a batch of HE multiplies of mixed N and CRT depth: one launch each ---
    mixed = None
    try:
        from cuyashe_gb300.api import MixedPlan

        mq = {62: 4611686018427322369, 127: Q_YASHE,
              190: 1569275433846670190958947355801916604025588861116000698369}
        rngm = np.random.default_rng(9)
        specs = [(int(rngm.choice([1024, 2048, 4096, 8192])), int(rngm.choice([62, 127, 190]))) for _ in range(512)]
        groups = {}
        for (n_, b_) in specs:
            groups.setdefault((n_, b_), 0)
            groups[(n_, b_)] += 1
        rings, bufs, jobs = {}, {}, []
        for (n_, b_), cnt in groups.items():
            Rm = cy.Ring(n_, mq[b_])
            lm = Rm.L
            hi_bits = (b_ - 1) - 64 * (lm - 1)  # values below 2^(b-1) < q
            raw = rngm.integers(0, 2**63, size=(2, cnt, n_, lm), dtype=np.uint64)
            raw[..., lm - 1] &= np.uint64((1 << hi_bits) - 1)
            if lm > 1:
                raw[..., :lm - 1] = rngm.integers(0, 2**64, size=(2, cnt, n_, lm - 1), dtype=np.uint64)
            Am = torch.from_numpy(raw[0].view(np.int64)).cuda()
            Bm = torch.from_numpy(raw[1].view(np.int64)).cuda()
            Cm = Rm.empty(cnt)
            rings[(n_, b_)], bufs[(n_, b_)] = Rm, (Am, Bm, Cm)
            for j in range(cnt):
                jobs.append(("mul", Rm, Am[j:j + 1], Bm[j:j + 1], Cm[j:j + 1]))
        order = list(range(len(jobs)))
        rngm.shuffle(order)
        jobs = [jobs[i] for i in order]
        plan = MixedPlan(jobs)  # sized and uploaded once; launches allocate nothing
        sched = plan.autotune()
        plan.launch()
        plan.status()
        ref = {key: bufs[key][2].clone() for key in bufs}

        def grouped():
            for key, Rm in rings.items():
                Am, Bm, Cm = bufs[key]
                Rm.polymul(Am, Bm, out=Cm)

        grouped()
        torch.cuda.synchronize()
        same = all(torch.equal(ref[key], bufs[key][2]) for key in bufs)
        msteps = max(5, args.steps // 4)
        t_one = time_steps(lambda: plan.launch(), msteps, stream)
        plan.status()
        g_mix = plan.graph()
        t_graph = time_steps(lambda: g_mix.launch(stream), msteps, stream)
        t_grp = time_steps(grouped, msteps, stream)
        mixed = {"products": len(jobs), "classes": len(groups), "schedule": sched,
                 "one_launch_products_per_s": len(jobs) * msteps / (t_one / 1000.0),
                 "graph_products_per_s": len(jobs) * msteps / (t_graph / 1000.0),
                 "per_ring_products_per_s": len(jobs) * msteps / (t_grp / 1000.0),
                 "one_launch_matches_per_ring": bool(same)}
        del plan, g_mix

        # HE multiplies (relinearised) of four (N, q, t) classes in one launch
        he_classes = [(2048, mq[62], 17), (4096, mq[127], 1024), (8192, mq[190], 65537), (1024, mq[190], 65537)]
        he_jobs, he_groups, he_msgs = [], [], []
        per_cls = 64
        for k_, (n_, q_, t_) in enumerate(he_classes):
            Yc = cy.Yashe(n_, q_, t_)
            Yc.keygen(500 + k_)
            pool = 4
            hm = torch.from_numpy(rngm.integers(0, t_, size=(2 * pool, n_), dtype=np.int64)).cuda()
            ct = Yc.encrypt(hm, seed=700 + k_)
            hi1 = torch.arange(per_cls, device="cuda") % pool
            hi2 = pool + (torch.arange(per_cls, device="cuda") * 3) % pool
            C1c, C2c = ct[hi1].contiguous(), ct[hi2].contiguous()
            Oc = Yc.ring.empty(per_cls)
            he_groups.append((Yc, C1c, C2c, Oc))
            he_msgs.append((hm, hi1, hi2))
            for j in range(per_cls):
                he_jobs.append(("yashe", Yc, C1c[j:j + 1], C2c[j:j + 1], Oc[j:j + 1], True))
        order = list(range(len(he_jobs)))
        rngm.shuffle(order)
        he_jobs = [he_jobs[i] for i in order]
        hplan = MixedPlan(he_jobs)
        hsched = hplan.autotune()
        hplan.launch()
        hplan.status()
        he_ref = [o.clone() for (_, _, _, o) in he_groups]

        def he_grouped():
            for Yc, C1c, C2c, Oc in he_groups:
                Yc.mul(C1c, C2c, relin=True, out=Oc)

        he_grouped()
        torch.cuda.synchronize()
        he_same = all(torch.equal(r_, g_[3]) for r_, g_ in zip(he_ref, he_groups))
        # decryption of the one-launch results of every class
        he_dec = True
        for (Yc, _, _, _), (hm, hi1, hi2), r_ in zip(he_groups, he_msgs, he_ref):
            got = Yc.decrypt(r_[:2]).cpu().numpy().view(np.uint64)
            PT = cy.Ring(Yc.n, Yc.t)
            exp = PT.polymul(PT.upload(hm[hi1[:2]].cpu().numpy().astype(object).tolist()),
                             PT.upload(hm[hi2[:2]].cpu().numpy().astype(object).tolist()))
            he_dec = he_dec and bool((got == exp.cpu().numpy().view(np.uint64)[..., 0]).all())
        t_he = time_steps(lambda: hplan.launch(), msteps, stream)
        hplan.status()
        g_he = hplan.graph()
        t_he_graph = time_steps(lambda: g_he.launch(stream), msteps, stream)
        t_he_grp = time_steps(he_grouped, msteps, stream)
        nhe = len(he_jobs)
        mixed["he_multiplies"] = {
            "jobs": nhe, "classes": ["%d/%d/t=%d" % (n_, q_.bit_length(), t_) for n_, q_, t_ in he_classes],
            "schedule": hsched,
            "one_launch_he_mults_per_s": nhe * msteps / (t_he / 1000.0),
            "graph_he_mults_per_s": nhe * msteps / (t_he_graph / 1000.0),
            "per_context_he_mults_per_s": nhe * msteps / (t_he_grp / 1000.0),
            "one_launch_over_per_context": t_he_grp / t_he,
            "one_launch_matches_per_context": bool(he_same), "decrypt_ok": bool(he_dec)}
        del hplan, g_he
        log("mixed batch:", mixed)
    except Exception as e:  # reported, not fatal for the headline
        log("mixed batch failed:", e)

    # ---- GPU encryption (on-device sampling) and decryption of the batch ---------
    crypt = None
    try:
        MSG = torch.from_numpy(np.ascontiguousarray(m1[idx1]).view(np.int64)).cuda()
        CT = Y.ring.empty(B)
        Y.encrypt(MSG, seed=5, out=CT)
        DEC = Y.decrypt(CT)
        torch.cuda.synchronize()
        enc_ok = torch.equal(DEC, MSG)
        enc_ms = time_steps(lambda: Y.encrypt(MSG, seed=6, out=CT), max(3, args.steps // 4), stream)
        dec_ms = time_steps(lambda: Y.decrypt(CT), max(3, args.steps // 4), stream)
        reps = max(3, args.steps // 4)
        crypt = {"encrypt_per_s": B * reps / (enc_ms / 1000.0), "decrypt_per_s": B * reps / (dec_ms / 1000.0),
                 "batch": B, "decrypt_of_encrypt_ok": bool(enc_ok)}
        log("encrypt/decrypt:", crypt)
    except Exception as e:
        log("encrypt bench failed:", e)

    # ---- deep level: N = 16384, 380-bit q, 64 pairs ------------------------------
    deep = None
    if not args.no_deep:
        try:
            deep = deep_bench(cy, max(3, args.steps // 2), stream)
            log("deep:", deep)
        except Exception as e:
            log("deep bench failed:", e)

    # ---- serving: Poisson arrivals of mixed-size multiplies --------------------
    serving = None
    if not args.no_serving:
        try:
            # 3 s of arrivals (60k requests): one host stall of tens of milliseconds on a
            # shared machine then touches well under 1% of the requests
            serving = serving_bench(cy, seconds=3.0)
            log("serving:", serving)
        except Exception as e:
            log("serving bench failed:", e)

    # ---- CPU baseline: the reference's multiply on the host cores ---------------
    cpu = None
    try:
        threads = os.cpu_count() or 1
        F, H, EV = Y.get_keys()
        pairs = 8 * threads  # about 20 s of CPU work on a 16-core Grace
        h1 = C1[:pairs].cpu().numpy().view(np.uint64)
        h2 = C2[:pairs].cpu().numpy().view(np.uint64)
        rate, secs = cpu_yashe_rate(pairs, threads, h1, h2, EV)
        cpu = {"value": rate, "unit": "HE mults/s", "cores": threads, "kind": "port",
               "sample": "%d HE multiplies at N=4096 with the reference's CPU multiply (C restatement), "
                         "%.1f s wall on %d threads" % (pairs, secs, threads)}
    except Exception as e:  # the baseline must not sink the GPU number
        log("cpu baseline failed:", e)

    clk = clocks.summary()
    try:
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        int_roof = int_roofline(kernels, counts, B, clk.get("sm_mhz") or 0.0, sms, ms_max / args.steps)
    except Exception as e:
        log("integer roofline failed:", e)
        int_roof = None
    line = {
        "metric": METRIC, "value": value, "unit": "HE mults/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "yashe_mul_relin N=4096 log2q=127 t=1024 w=2^32 ell=%d" % info.ell,
                   "batch_pairs_per_gpu": B, "tensor_primes": info.tensor_primes, "relin_primes": info.relin_primes,
                   "l2": "inputs larger than L2 (%.0f MB per step)" % (2 * B * CT_BYTES / 1e6),
                   "parallelism": "replicas x%d" % world, "schedules": tuning},
        "clocks": clk,
        "e2e": {"value": e2e_rate, "unit": "HE mults/s", "h2d_bytes_per_step": 2 * B * CT_BYTES,
                "d2h_bytes_per_step": B * CT_BYTES, "output_matches_device": e2e_ok,
                "api": "cy_yashe_mul_host (page-locked host buffers, host wall clock)", "copy_alone": copy_gbs,
                "windows_per_s": [round(w) for w in e2e_windows], "calls_per_window": e2e_per_window,
                "statistic": "median of the windows"},
        "gpu_launches": launches,
        "roofline": roofline,
        "int_roofline": int_roof,
        "step_roofline": {"bound": "hbm", "achieved": round(step_gbs, 1), "peak": peak, "unit": "GB/s",
                          "frac": round(step_gbs / peak, 4), "algorithmic_bytes_per_step": step_bytes},
        "kernels": kernels,
        "plain_per_call": {"he_mults_per_s": plain_rate, "batched_over_plain": value / world / plain_rate},
        "polymul": {"batched_per_s": poly_rate, "plain_per_call_per_s": poly_plain,
                    "batched_over_plain": poly_rate / poly_plain, "q_bits": 127, "batch": PB,
                    "e2e_per_s": poly_e2e, "e2e_matches_device": poly_e2e_ok,
                    "e2e_api": "cy_polymul_host (page-locked host buffers)"},
        "mixed_batch": mixed,
        "gpu_encrypt_decrypt": crypt,
        "ntt_standalone": ntt_line,
        "deep_level": deep,
        "cuda_graph": graphs,
        "serving": serving,
        "decrypt_check": decrypt_ok,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    replicas.close(rep)


def ncu_schedules(batch: int = 1024, only: str = "all"):
    """One call of every N = 4096 schedule of the product (plain and centred),
    the keyswitch and the standalone NTT (forced with cy_tuning_import) between
    cudaProfilerStart/Stop, for ncu's per-schedule counts; prints the order.
    `ksm=v` runs keyswitch schedule v inside an HE multiply of one chunk (170
    pairs: the tensor residues of 24 MiB), where its input is limb-major; a
    capture filtered to k_keyswitch then has one launch per such schedule.
    `only`: "all", or a comma-separated list such as "mulc=7,ks=5,ntt=9"."""
    import numpy as np
    import torch

    import cuyashe_gb300 as cy

    cy.lib()

    def variants(op):
        out = []
        for v in range(64):
            try:
                cy.tuning_import("n%d.l2.%s=%d" % (N, op, v))
            except cy.CyError:
                break
            out.append(v)
        return out

    Y = cy.Yashe(N, Q_YASHE, T, W_BITS, 8.0)
    Y.keygen(1)
    R = cy.Ring(N, Q_POLY)
    rng = np.random.default_rng(5)
    A = torch.from_numpy(rng.integers(0, 2**63, size=(batch, N, L), dtype=np.uint64).view(np.int64)).cuda()
    A[..., 1] &= (1 << 62) - 1  # < 2^126 < q
    Bt = A.flip(0).contiguous()
    O = Y.ring.empty(batch)
    RES = torch.zeros((batch, R.k, N), dtype=torch.int32, device="cuda")
    plan = [(op, v) for op in ("mul", "mulc", "ks", "ntt") for v in variants(op)]
    plan += [("ksm", v) for v in variants("ks")]
    KSM = 170
    if only != "all":
        want = {tuple(x.split("=")) for x in only.split(",")}
        plan = [(op, v) for op, v in plan if (op, str(v)) in want]

    def run(op, v):
        cy.tuning_import("n%d.l2.%s=%d" % (N, "ks" if op == "ksm" else op, v))
        if op == "mul":
            R.polymul(A, Bt, out=O)
        elif op == "mulc":
            Y.mul(A, Bt, relin=False, out=O)
        elif op == "ks":
            Y.keyswitch(A, out=O)
        elif op == "ksm":
            Y.mul(A[:KSM], Bt[:KSM], relin=True, out=O[:KSM])
        else:
            R.ntt(RES)
            R.ntt(RES, inverse=True)

    for op, v in plan:
        run(op, v)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for op, v in plan:
        run(op, v)
        torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print("ORDER", ";".join("%s=%d" % p for p in plan), flush=True)


def _free_port() -> int:
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def launch_ranks(args, argv):
    """`--gpus N` (N > 1) outside a launcher: start N ranks of this script with
    torch.distributed.run on this node (one replica per GPU) and return their
    exit status; None when this process already is a rank or N == 1."""
    if args.gpus <= 1 or "WORLD_SIZE" in os.environ:
        return None
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.abspath(__file__)] + argv
    log("launching %d ranks:" % args.gpus, " ".join(cmd))
    return subprocess.call(cmd)


def cpu_dry_run(args):
    """The replica bookkeeping of a run without CUDA (gloo): every rank takes its
    contiguous share of the job's pairs, times a stand-in step, and rank 0 prints
    one line with the world size and every rank's share. For tests of the
    launcher; no GPU figure is measured."""
    from cuyashe_gb300 import replicas

    rep = replicas.from_env("gloo")
    total = rep.world * args.batch
    start, stop = replicas.shard(total, rep.rank, rep.world)
    replicas.barrier(rep)
    t0 = time.perf_counter()
    acc = 0
    for _ in range(args.steps):
        acc += sum(range(start, stop))  # stand-in work on this rank's share
    ms = (time.perf_counter() - t0) * 1000.0
    ms_max = replicas.max_over_ranks(rep, ms)
    units = replicas.sum_over_ranks(rep, stop - start)
    if rep.is_root:
        line = {"metric": METRIC, "value": None, "unit": "HE mults/s", "n_gpus": rep.world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / max(1, args.steps), "higher_is_better": True,
                "scaling": "weak", "dry_run": True, "pairs_per_step": int(units),
                "shards": [list(replicas.shard(total, r, rep.world)) for r in range(rep.world)],
                "config": {"workload": "yashe_mul_relin N=4096 log2q=127 t=1024 w=2^32 ell=4",
                           "batch_pairs_per_gpu": args.batch, "parallelism": "replicas x%d" % rep.world}}
        print(json.dumps(line), flush=True)
    replicas.close(rep)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=4096, help="ciphertext pairs per GPU per step")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default NTT schedules")
    ap.add_argument("--schedules", default="", metavar="TUNING",
                    help="schedules to use instead of autotuning (cy_tuning_export format)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-deep", action="store_true", help="skip the N=16384 / 380-bit measurement")
    ap.add_argument("--serving-only", type=float, default=0.0, metavar="SECONDS",
                    help="run only the serving measurement over SECONDS of arrivals and print it")
    ap.add_argument("--ncu-step", action="store_true",
                    help="set up, warm up, run one step inside cudaProfilerStart/Stop, exit (for ncu)")
    ap.add_argument("--ncu-deep", type=int, default=0, metavar="PAIRS",
                    help="the same for one autotuned deep-level step (N=16384, 380-bit q) of PAIRS pairs")
    ap.add_argument("--ncu-schedules", nargs="?", const="all", default=None, metavar="LIST",
                    help="one call of every N=4096 schedule (or of LIST, e.g. mulc=7,ks=5,ntt=9) inside "
                         "cudaProfilerStart/Stop, exit (for ncu)")
    ap.add_argument("--cpu-dry-run", action="store_true",
                    help="ranks and shares only, without CUDA (tests of the multi-GPU launcher)")
    args = ap.parse_args()
    rc = launch_ranks(args, sys.argv[1:])
    if rc is not None:
        sys.exit(rc)
    if args.cpu_dry_run:
        cpu_dry_run(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        log("note: warm-up raised to 3")
        args.warmup = 3
    if args.ncu_schedules is not None:
        ncu_schedules(only=args.ncu_schedules)
    elif args.impl == "reference":
        run_reference(args)
    elif args.serving_only > 0:
        import cuyashe_gb300 as cy

        cy.lib()
        print(json.dumps(serving_bench(cy, seconds=args.serving_only)), flush=True)
    elif args.ncu_deep > 0:
        ncu_deep_step(args.ncu_deep)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
