"""Serving: the continuous-batching request loop (lsgb_server_* in include/lsgb.h).

``Server`` wraps the native loop: ``submit`` one object at a time as it arrives,
``poll`` completed (id, best index, best power, submit time, completion time).
``replay`` drives a ``synth.Stream`` in real time -- each object is submitted at its
Poisson arrival time -- and reports p50/p99 latency (submit to completion) next to
throughput. The batching, admission and device work all happen in the native
dispatcher thread; Python only feeds arrivals and collects results.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from . import _native, synth
from .engine import GENERALIZED, STANDARD, LsgbError, _precision

_dp = ctypes.POINTER(ctypes.c_double)


class Server:
    def __init__(self, n_freq: int, fmin: float, df: float, variant: int = STANDARD,
                 precision="mixed", normalize: bool = True, slots: int = 3,
                 max_batch: int = 4096, hbm_budget_bytes: int = 4 << 30, device: int = 0):
        self._lib = _native.lsgb()
        h = ctypes.c_void_p()
        rc = self._lib.lsgb_server_create(device, variant, _precision(precision), float(fmin),
                                          float(df), int(n_freq), int(bool(normalize)),
                                          int(slots), int(max_batch), int(hbm_budget_bytes),
                                          ctypes.byref(h))
        if rc != 0:
            raise LsgbError(rc, self._lib.lsgb_last_error().decode())
        self._h = h
        self.variant = variant

    def submit(self, obj_id: int, t, y, dy=None):
        t = np.ascontiguousarray(t, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        dyp = None
        if self.variant == GENERALIZED:
            dy = np.ascontiguousarray(dy, dtype=np.float64)
            dyp = dy.ctypes.data_as(_dp)
        rc = self._lib.lsgb_server_submit(self._h, int(obj_id), t.ctypes.data_as(_dp),
                                          y.ctypes.data_as(_dp), dyp, t.size)
        if rc != 0:
            raise LsgbError(rc, self._lib.lsgb_last_error().decode())

    def poll(self, max_items: int = 1 << 16):
        ids = np.empty(max_items, np.uint64)
        idx = np.empty(max_items, np.uint32)
        pw = np.empty(max_items, np.float64)
        ts = np.empty(max_items, np.float64)
        td = np.empty(max_items, np.float64)
        n = self._lib.lsgb_server_poll(
            self._h, max_items, ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            idx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), pw.ctypes.data_as(_dp),
            ts.ctypes.data_as(_dp), td.ctypes.data_as(_dp))
        if n < 0:
            raise LsgbError(n, self._lib.lsgb_last_error().decode())
        return ids[:n], idx[:n], pw[:n], ts[:n], td[:n]

    def stats(self):
        out = (ctypes.c_uint64 * 5)()
        self._lib.lsgb_server_stats(self._h, out)
        keys = ("batches", "objects_done", "largest_batch", "waiting", "peak_inflight_bytes")
        return dict(zip(keys, (int(v) for v in out)))

    def peaks(self):
        out = (ctypes.c_uint64 * 4)()
        self._lib.lsgb_server_peaks(self._h, out)
        keys = ("peak_inflight_bytes", "peak_slots_in_flight", "peak_waiting", "budget_deferrals")
        return dict(zip(keys, (int(v) for v in out)))

    def now(self) -> float:
        return float(self._lib.lsgb_server_now())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lsgb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def replay(stream: synth.Stream, n_objects: int | None = None, variant: int = STANDARD,
           precision="mixed", slots: int = 3, max_batch: int = 4096,
           hbm_budget_bytes: int = 4 << 30, objects=None):
    """Submit stream objects at their arrival times; return the latency report and results.

    ``objects``: optional pre-generated list of (t, y, dy); default draws them from
    the stream (``synth.stream_object``) before the clock starts.
    """
    n = stream.size.size if n_objects is None else min(int(n_objects), stream.size.size)
    fmin, fmax, nf = stream.fmin, stream.fmax, stream.n_freq
    df = (fmax - fmin) / nf
    if objects is None:
        objects = []
        for i in range(n):
            t, y = synth.stream_object(stream, i)
            objects.append((t, y, np.ones_like(t)))
    srv = Server(nf, fmin, df, variant=variant, precision=precision, normalize=True, slots=slots,
                 max_batch=max_batch, hbm_budget_bytes=hbm_budget_bytes)
    # warm the engines (first launches pay module loading) outside the measured stream
    for k in range(slots):
        t, y, dy = objects[k % n]
        srv.submit(10 ** 12 + k, t, y, dy)
    while len(srv.poll()[0]) == 0:
        time.sleep(1e-3)
    time.sleep(0.05)
    srv.poll()

    results = []
    collected = [0]
    done = threading.Event()

    def collector():
        while not done.is_set():
            r = srv.poll()
            keep = r[0] < n  # warm-up objects finishing late are not part of the stream
            if keep.any():
                results.append(tuple(x[keep] for x in r))
                collected[0] += int(keep.sum())
            elif not len(r[0]):
                time.sleep(2e-4)

    th = threading.Thread(target=collector, daemon=True)
    th.start()
    lateness = np.zeros(n)
    t0 = time.perf_counter()
    c0 = srv.now()
    for i in range(n):
        target = t0 + stream.arrival[i] - stream.arrival[0]
        while True:
            d = target - time.perf_counter()
            if d <= 0:
                break
            if d > 3e-4:
                time.sleep(d - 2e-4)
        lateness[i] = time.perf_counter() - target
        t, y, dy = objects[i]
        srv.submit(i, t, y, dy)
    # every submitted object is collected before the loop is shut down (results still
    # queued in the server when it is destroyed would be discarded)
    deadline = time.perf_counter() + 60.0
    while collected[0] < n and time.perf_counter() < deadline:
        time.sleep(1e-3)
    wall = time.perf_counter() - t0
    done.set()
    th.join()
    stats_before_close = {**srv.stats(), **srv.peaks()}
    srv.close()
    ids = np.concatenate([r[0] for r in results]) if results else np.zeros(0, np.uint64)
    order = np.argsort(ids)
    cat = lambda k: np.concatenate([r[k] for r in results])[order]
    idx, pw, ts, td = cat(1), cat(2), cat(3), cat(4)
    ids = ids[order]
    lat = td - ts
    pairs = float(np.sum(stream.size[:n])) * nf
    report = {
        "objects": int(n), "completed": int(ids.size), "rate_hz": float(
            (n - 1) / (stream.arrival[n - 1] - stream.arrival[0])) if n > 1 else None,
        "n_freq": int(nf), "latency_p50_ms": float(np.percentile(lat, 50) * 1e3),
        "latency_p99_ms": float(np.percentile(lat, 99) * 1e3),
        "latency_max_ms": float(lat.max() * 1e3), "latency_mean_ms": float(lat.mean() * 1e3),
        "submit_lateness_p99_ms": float(np.percentile(lateness, 99) * 1e3),
        "wall_s": wall, "pairs_per_s": pairs / wall,
        "busy_span_s": float(td.max() - c0) if td.size else None,
        "slots": slots, "max_batch": max_batch, "hbm_budget_bytes": int(hbm_budget_bytes),
        **{k: v for k, v in stats_before_close.items() if k != "objects_done"},
    }
    return report, {"ids": ids, "best_idx": idx, "best_power": pw, "latency_s": lat}
