#!/usr/bin/env python
"""Throughput of the Lomb-Scargle hot path on one GB300, one JSON line on stdout.

Workload (the reference's headline batch): 999 objects with log-normal observation
counts (round(LogNormal(ln 150, 0.6)) clipped to [20, 1500], ~176k rows, seeded,
synthetic), standard L-S, 1e6 angular frequencies in [1.005, 150.796). One step =
one batch periodogram with the fused per-object argmax, mixed precision form, inputs
resident in HBM, replayed from a CUDA-graph plan (lsgb_plan_launch), in the engine's
default form (the tensor-core form: split-FP16 tcgen05 MMAs, FP32 accumulation and folds,
FP64 phase anchors). Metric: observation x frequency pairs per second.

Also reported on the same line:
  plain_fp64   the FP64 drop-in form on the first frequencies of the same grid;
  e2e          the engine's host-buffer C ABI (lsgb_periodogram_host): pinned host
               inputs in, best index/power out, copies inside the timed region;
  e2e_dropin   LombScarglePy of libpylsnoerrorfloat.so (MODE 1) returning the full
               periodogram to a host buffer, as source/lombscarglegpu.py calls it;
  roofline     the tensor kernel's FP16 MMA flops (48 per pair, standard variant) per
               second against the measured dense bf16/FP16 tensor peak
               (MEASURED_PEAKS.json, burst);
  cuda_core_form  the same batch in the CUDA-core mixed form (FP32 second-order recurrence),
               with its FP32-pipe ops per pair against the FP32 FMA peak measured in the
               same run (cuBLAS SGEMM, TF32 off);
  cpu_baseline the FP64 oracle (the reference's CPU algorithm) on all host cores;
  clocks       nvidia-smi samples taken during the timed region (every 50 ms), and, under
               sustained_load_window, during a further second of the same replays, untimed;
  serving      the continuous-batching loop on a Poisson stream (100,000 objects at
               2,000/s, 2e5 frequencies): p50 / p99 latency and throughput.
`--impl reference` runs the reference arm: the reference's CPU algorithm on the
host cores (its own build when it is present, else the oracle port).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "obs x freq pairs/s (mixed form, 1 GB300)"
UNIT = "pairs/s"
# tensor form, standard variant: two complex products (v e^ia x e^imb, e^2ia x e^2imb),
# each 4 real MACs x 3 split-FP16 products = 24 MACs = 48 flops per (obs, freq) pair; the
# algorithm itself needs 16 of them (the x3 buys FP32 accuracy from FP16 operands).
# Generalized: three complex products (two weight groups at phase 0), 72 and 24 flops.
TENSOR_FLOPS_PER_PAIR_STD = 48
TENSOR_FLOPS_PER_PAIR_GEN = 72
ALGORITHMIC_FLOPS_PER_PAIR_STD = 16
ALGORITHMIC_FLOPS_PER_PAIR_GEN = 24
# CUDA-core form 2 (F = 12): per observation and thread 4 (odd-lane offset) + 8 (rotation
# to the second pair) + 4 x 4 (second-order steps) + 6 x 8 (accumulations) = 76 FP32-pipe
# lane-ops for 12 pairs
CUDA_CORE_SHAPE_STD = (12, 256, 2, 2, 0)
OPS_PER_PAIR_CUDA_CORE = 76 / 12
# DRAM read + write bytes of one tensor-kernel launch, from an ncu capture of the same
# batch at 1e5 frequencies (dram__bytes_read.sum + dram__bytes_write.sum): the operand
# table (32 KB of split-FP16 left operands per K-block, 11,487 K-blocks: 376 MB) is read
# from DRAM once per launch whatever the grid size, because the units of one object run
# back to back and re-read it from L2; nothing is written without a periodogram
TENSOR_DRAM_BYTES_PER_LAUNCH = 3.84e8
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_BF16_TFLOPS = 1900.0
L2_FLUSH_BYTES = 256 << 20


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(
        os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, interval_ms: int = 50):
        self.device = device
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def tensor_peak_tflops():
    """(peak TFLOP/s, source) of dense bf16/FP16 MMA: the burst figure measured on this
    GPU model (MEASURED_PEAKS.json), else the fallback."""
    try:
        d = json.loads(MEASURED_PEAKS.read_text())
        return float(d["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (burst), of measured"
    except (OSError, ValueError, KeyError):
        return FALLBACK_BF16_TFLOPS, "fallback 1.9 PFLOP/s bf16 burst, of fallback"


def fp32_peak_ops(torch, dev):
    """FP32 FMA throughput of cuBLAS SGEMM (TF32 off), in FMA ops/s, best of 5."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        for _ in range(2):
            torch.mm(a, b)
        best = 1e30
        for _ in range(5):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.mm(a, b)
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e) / 1e3)
        return n ** 3 / best
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def cpu_baseline(w, n_freq_sample: int):
    """The FP64 oracle (reference CPU algorithm) on the first n_freq_sample frequencies."""
    from oracle import pyoracle

    ws = w.subset_freqs(n_freq_sample)
    t0 = time.perf_counter()
    pyoracle.batch_pgram(0, ws.t, ws.y, None, ws.offsets, ws.fmin, ws.df, n_freq=ws.n_freq)
    dt = time.perf_counter() - t0
    return {"value": ws.pairs / dt, "unit": UNIT, "cores": pyoracle.max_threads(), "kind": "port",
            "sample": f"{w.n_obj} objects x first {n_freq_sample} of {w.n_freq} frequencies "
                      f"({ws.pairs:.3g} pairs, {dt:.2f} s)"}


def measure_config(eng, torch, dev, stream, flush, w, variant, err_freqs):
    """One more benchmark workload through the default mixed form: kernel time (median of
    runs after a first one), pairs/s, the tensor-pipe roofline, and its largest absolute
    difference from the plain FP64 form (the drop-in arithmetic, itself pinned to the FP64
    oracle by the tests) on the first err_freqs frequencies, with the best frequencies of
    both forms compared there."""
    t = torch.from_numpy(w.t).to(dev)
    y = torch.from_numpy(w.y).to(dev)
    dy = torch.from_numpy(w.dy).to(dev) if variant else None
    bi = torch.empty(w.n_obj, dtype=torch.int32, device=dev)
    bp = torch.empty(w.n_obj, dtype=torch.float64, device=dev)
    ms = []
    for _ in range(3):
        flush.zero_()
        eng.run_device(variant, "mixed", t, y, dy, w.offsets, w.fmin, w.df, w.n_freq,
                       variant == 0, None, bi, bp, stream)
        ms.append(eng.last_kernel_ms())
    kms = float(np.median(ms[1:]))
    peak_tf, peak_src = tensor_peak_tflops()
    fpp = TENSOR_FLOPS_PER_PAIR_GEN if variant else TENSOR_FLOPS_PER_PAIR_STD
    afpp = ALGORITHMIC_FLOPS_PER_PAIR_GEN if variant else ALGORITHMIC_FLOPS_PER_PAIR_STD
    achieved = w.pairs * fpp / (kms / 1e3) / 1e12
    ws = w.subset_freqs(min(err_freqs, w.n_freq))
    pgs = {}
    for form in ("mixed", "plain"):
        pg = torch.empty((ws.n_obj, ws.n_freq), dtype=torch.float64, device=dev)
        eng.run_device(variant, form, t, y, dy, ws.offsets, ws.fmin, ws.df, ws.n_freq,
                       variant == 0, pg, None, None, stream)
        pgs[form] = pg
    torch.cuda.synchronize()
    diff = float((pgs["mixed"] - pgs["plain"]).abs().max().item())
    km = pgs["mixed"].argmax(dim=1)
    kp = pgs["plain"].argmax(dim=1)
    rows = torch.arange(ws.n_obj, device=dev)
    gap = (pgs["plain"][rows, kp] - pgs["plain"][rows, km]).cpu().numpy()
    same = int((km == kp).sum().item())
    ties = int(((km != kp).cpu().numpy() & (gap <= 1e-4)).sum())
    del pgs
    return {"value": w.pairs / (kms / 1e3), "unit": UNIT, "kernel_ms": kms,
            "pairs": w.pairs, "n_obj": w.n_obj, "rows": w.n_rows, "n_freq": w.n_freq,
            "variant": "generalized" if variant else "standard",
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak_tf,
                         "unit": "TFLOP/s", "frac": achieved / peak_tf, "peak_source": peak_src,
                         "flops_per_pair": fpp, "algorithmic_flops_per_pair": afpp},
            "max_abs_err_vs_plain_fp64": diff,
            "error_sample": f"first {ws.n_freq} frequencies, all {ws.n_obj} objects",
            "best_identical": same, "best_within_1e-4_tie": ties,
            "best_other": ws.n_obj - same - ties}


def reference_arm(args):
    """The reference's CPU path on this host (all cores), bounded sample per step."""
    from gpu_lomb_scargle_gb300 import synth

    rank, world, _ = rank_info()
    if rank != 0:
        return
    w = synth.lognormal_batch()
    nf = args.ref_freqs
    ws = w.subset_freqs(nf)
    kind, cores = "port", None
    ref_lib = ROOT / "oracle" / "_ref" / "libpylsnoerrordouble.so"
    run = None
    try:
        import ctypes
        lib = ctypes.CDLL(str(ref_lib))
        arr = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        uarr = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
        lib.LombScarglePy.argtypes = [uarr, arr, arr, arr, ctypes.c_uint, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_uint, ctypes.c_int, arr]
        pg = np.zeros(ws.n_obj * nf)
        ids = np.ascontiguousarray(ws.obj_id, np.uint32)
        dy = np.ones(ws.n_rows)
        import tempfile
        tmp = tempfile.mkdtemp()

        def run():
            cwd = os.getcwd()
            os.chdir(tmp)
            try:
                lib.LombScarglePy(ids, ws.t, ws.y.copy(), dy, ws.n_rows, ws.fmin, ws.fmax, nf, 4, pg)
            finally:
                os.chdir(cwd)
        kind, cores = "reference", os.cpu_count()
    except OSError:
        from oracle import pyoracle

        def run():
            pyoracle.batch_pgram(0, ws.t, ws.y, None, ws.offsets, ws.fmin, ws.df, n_freq=nf)
        cores = pyoracle.max_threads()
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    os.dup2(devnull, 1)  # the reference library prints progress to stdout
    try:
        for _ in range(args.warmup):
            run()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        dt = (time.perf_counter() - t0) / args.steps
    finally:
        sys.stdout.flush()
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)
    value = ws.pairs / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded log-normal batch, stands in for the reference's missing "
                    "999-object file)",
            "config": {"workload": "lognormal_999obj_1e6freq_standard", "n_obj": w.n_obj,
                       "rows": w.n_rows, "n_freq": w.n_freq, "sample_freqs": nf},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"{w.n_obj} objects x first {nf} of {w.n_freq} frequencies "
                                       f"per step ({ws.pairs:.3g} pairs)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lsgb", choices=["lsgb", "reference"])
    ap.add_argument("--n-freq", type=int, default=1_000_000)
    ap.add_argument("--plain-freqs", type=int, default=20_000,
                    help="frequencies of the plain FP64 comparison (0 = skip)")
    ap.add_argument("--cpu-freqs", type=int, default=10_000,
                    help="frequencies of the CPU-baseline sample (0 = skip)")
    ap.add_argument("--ref-freqs", type=int, default=2_000,
                    help="frequencies per step of the reference arm")
    ap.add_argument("--no-dropin", action="store_true")
    ap.add_argument("--serve-objects", type=int, default=100_000,
                    help="objects of the Poisson serving replay (0 = skip)")
    ap.add_argument("--configs", type=int, default=1,
                    help="also measure the single-object, generalized and long-object "
                         "workloads (0 = skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)

    import torch

    from gpu_lomb_scargle_gb300 import engine as E
    from gpu_lomb_scargle_gb300 import synth

    rank, world, local = rank_info()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    # weak scaling: every rank owns its own batch of the same shape
    w = synth.lognormal_batch(seed=2000 + rank, n_freq=args.n_freq)
    eng = E.Engine(local)
    t = torch.from_numpy(w.t).to(dev)
    y = torch.from_numpy(w.y).to(dev)
    bi = torch.empty(w.n_obj, dtype=torch.int32, device=dev)
    bp = torch.empty(w.n_obj, dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    # the timed steps replay a CUDA-graph plan of the batch (one cudaGraphLaunch per step)
    plan = eng.plan(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, True, None, bi, bp)
    kernels_per_step = plan.info()[0]

    for _ in range(args.warmup):
        plan.launch(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kern_ms = []
    launches = 0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (outside the events)
            starts[i].record(stream)
            plan.launch(stream)
            ends[i].record(stream)
            kern_ms.append(plan.info(kernel_time=True)[2])
            launches += kernels_per_step
        torch.cuda.synchronize()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = float(np.mean(step_ms))
    if world > 1:
        from gpu_lomb_scargle_gb300 import shard
        ms = shard.max_over_ranks(ms)  # the slowest rank's step time
    value = w.pairs * world / (ms / 1e3)
    best_idx = bi.cpu().numpy()

    # e2e through the host-buffer C ABI with pinned inputs, on every rank at once (a barrier
    # before, the slowest rank's time after)
    th = torch.from_numpy(w.t).pin_memory().numpy()
    yh = torch.from_numpy(w.y).pin_memory().numpy()
    oi = torch.empty(w.n_obj, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    op = torch.empty(w.n_obj, dtype=torch.float64).pin_memory().numpy()
    offs = np.ascontiguousarray(w.offsets, np.uint64)  # the caller's row offsets, once
    for _ in range(2):
        eng.run_host(0, "mixed", th, yh, None, offs, w.fmin, w.df, w.n_freq, True,
                     out_idx=oi, out_power=op)
    if world > 1:
        torch.distributed.barrier()
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        eng.run_host(0, "mixed", th, yh, None, offs, w.fmin, w.df, w.n_freq, True,
                     out_idx=oi, out_power=op)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e_t))
    if world > 1:
        from gpu_lomb_scargle_gb300 import shard
        e2e_s = shard.max_over_ranks(e2e_s)
    e2e = {"value": w.pairs * world / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(th.nbytes + yh.nbytes + 8 * (w.n_obj + 1)),
           "d2h_bytes_per_step": int(oi.nbytes + op.nbytes),
           "api": "lsgb_periodogram_host (C ABI), pinned host buffers, best period per object"}
    if not np.array_equal(oi, best_idx.astype(np.uint32)):
        e2e["mismatch_vs_device_path"] = True

    if rank != 0:
        return
    clocks = clk.summary()
    # The timed region is short (tens of ms): the same replays, untimed, for about a second
    # more give the clocks under sustained load of this workload, reported apart.
    with ClockSampler(local) as clk2:
        t_end = time.perf_counter() + 1.0
        while time.perf_counter() < t_end:
            for _ in range(10):
                plan.launch(stream)
            torch.cuda.synchronize()
    clocks["sustained_load_window"] = clk2.summary()
    kms = float(np.mean(kern_ms))
    shape = eng.get_tuning(0)  # (F, threads, min CTAs, form, unroll)
    tensor_form = shape[3] == 3
    extra = {}
    peak_ops = fp32_peak_ops(torch, dev)
    if tensor_form:
        peak_tf, peak_src = tensor_peak_tflops()
        achieved = w.pairs * TENSOR_FLOPS_PER_PAIR_STD / (kms / 1e3) / 1e12
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                    "frac": achieved / peak_tf, "traffic": TENSOR_DRAM_BYTES_PER_LAUNCH,
                    "peak_source": peak_src, "flops_per_pair": TENSOR_FLOPS_PER_PAIR_STD,
                    "algorithmic_flops_per_pair": ALGORITHMIC_FLOPS_PER_PAIR_STD,
                    "algorithmic_frac": achieved / peak_tf * ALGORITHMIC_FLOPS_PER_PAIR_STD
                    / TENSOR_FLOPS_PER_PAIR_STD,
                    "kernel_ms": kms, "kernel": "tensor_kernel<standard> (lsgb_tensor.cu)"}
        # the CUDA-core form on the same batch, against the FP32 FMA peak
        saved = eng.get_tuning(0)
        eng.set_tuning(0, *CUDA_CORE_SHAPE_STD)
        try:
            cm = []
            for _ in range(3):
                flush.zero_()
                eng.run_device(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, True,
                               None, bi, bp, stream)
                cm.append(eng.last_kernel_ms())
        finally:
            eng.set_tuning(0, *saved)
        cms = float(np.median(cm[1:]))
        cach = w.pairs * OPS_PER_PAIR_CUDA_CORE / (cms / 1e3)
        extra["cuda_core_form"] = {
            "value": w.pairs / (cms / 1e3), "unit": UNIT, "kernel_ms": cms,
            "shape": list(CUDA_CORE_SHAPE_STD),
            "roofline": {"bound": "fp32", "achieved": cach / 1e12, "peak": peak_ops / 1e12,
                         "unit": "Tops/s (FP32 pipe ops)", "frac": cach / peak_ops,
                         "ops_per_pair": OPS_PER_PAIR_CUDA_CORE,
                         "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run"}}
    else:
        achieved = w.pairs * OPS_PER_PAIR_CUDA_CORE / (kms / 1e3)
        roofline = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak_ops / 1e12,
                    "unit": "Tops/s (FP32 pipe ops)", "frac": achieved / peak_ops, "traffic": None,
                    "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run",
                    "ops_per_pair": OPS_PER_PAIR_CUDA_CORE, "kernel_ms": kms}

    # the three best frequencies per object in the same kernel pass (source/main.cu:1165-1219)
    if tensor_form:
        ti = torch.empty((w.n_obj, 3), dtype=torch.int32, device=dev)
        tp = torch.empty((w.n_obj, 3), dtype=torch.float64, device=dev)
        tm = []
        for _ in range(3):
            flush.zero_()
            eng.run_device_top3(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, True,
                                None, ti, tp, stream)
            tm.append(eng.last_kernel_ms())
        top3_ms = float(np.median(tm[1:]))
        extra["top3"] = {"kernel_ms": top3_ms, "over_argmax": top3_ms / kms,
                         "first_equals_argmax": bool(np.array_equal(
                             ti[:, 0].cpu().numpy(), best_idx.astype(np.int32)))}

    # the other benchmark workloads (single object, generalized batch, long object)
    if tensor_form and args.configs and world == 1:
        extra["configs"] = {
            "single_3555obs_1e5freq_standard": measure_config(
                eng, torch, dev, stream, flush, synth.single_object(), 0, 100_000),
            "lognormal_999obj_1e6freq_generalized": measure_config(
                eng, torch, dev, stream, flush, synth.lognormal_batch_dmag(), 1, 3_000),
            "long_200kobs_1e7freq_standard": measure_config(
                eng, torch, dev, stream, flush, synth.long_object(), 0, 20_000),
        }

    # plain FP64 drop-in form on the first plain_freqs frequencies
    if args.plain_freqs and world == 1:
        wp = w.subset_freqs(args.plain_freqs)
        eng.run_device(0, "plain", t, y, None, wp.offsets, wp.fmin, wp.df, wp.n_freq, True, None,
                       bi, bp, stream)
        torch.cuda.synchronize()
        pm = []
        for _ in range(2):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.zero_()
            s.record(stream)
            eng.run_device(0, "plain", t, y, None, wp.offsets, wp.fmin, wp.df, wp.n_freq, True,
                           None, bi, bp, stream)
            e.record(stream)
            e.synchronize()
            pm.append(s.elapsed_time(e))
        pv = wp.pairs / (np.mean(pm) / 1e3)
        extra["plain_fp64"] = {"value": pv, "unit": UNIT, "ms_per_step": float(np.mean(pm)),
                               "sample": f"first {args.plain_freqs} frequencies of the same grid"}
        extra["mixed_over_plain"] = value / pv

    if not args.no_dropin and world == 1:
        from gpu_lomb_scargle_gb300 import lombscarglegpu as lsg
        lib = lsg._library(False, "float")
        t32 = np.ascontiguousarray(w.t, np.float32)
        y32 = np.ascontiguousarray(w.y, np.float32)
        ids = np.ascontiguousarray(w.obj_id, np.uint32)
        ones = np.ones(w.n_rows, np.float32)
        pg = np.empty(w.n_obj * w.n_freq, np.float32)
        pg.fill(0.0)  # touch every page now: first-touch faults are not the library's time
        dt = []
        devnull = os.open(os.devnull, os.O_WRONLY)
        saved = os.dup(1)
        sys.stdout.flush()
        os.dup2(devnull, 1)
        try:
            for i in range(9):
                t0 = time.perf_counter()
                lib.LombScarglePy(ids, t32, y32, ones, w.n_rows, w.fmin, w.fmax, w.n_freq, 1, pg)
                if i:  # the first call loads the library's kernels and sizes its buffers
                    dt.append(time.perf_counter() - t0)
        finally:
            sys.stdout.flush()
            os.dup2(saved, 1)
            os.close(saved)
            os.close(devnull)
        extra["e2e_dropin"] = {"value": w.pairs / float(np.median(dt)), "unit": UNIT,
                               "ms_per_call": [round(1e3 * x, 2) for x in dt],
                               "h2d_bytes_per_step": int(t32.nbytes * 3 + ids.nbytes),
                               "d2h_bytes_per_step": int(pg.nbytes),
                               "api": "LombScarglePy, libpylsnoerrorfloat.so, MODE 1, full pgram"}
        del pg

    if args.serve_objects and world == 1:
        from gpu_lomb_scargle_gb300 import serve
        plan.close()
        eng.close()
        torch.cuda.empty_cache()
        st = synth.stream(n_obj=args.serve_objects)
        rep, _ = serve.replay(st, slots=3, max_batch=4096, hbm_budget_bytes=4 << 30)
        rep["workload"] = (f"{st.size.size} objects, Poisson {2000} objects/s, sizes "
                           "round(LogNormal(ln 80, 0.8)) in [10, 1000], 2e5 frequencies, mixed form")
        extra["serving"] = rep
        extra["p50_latency_ms"] = rep["latency_p50_ms"]
        extra["p99_latency_ms"] = rep["latency_p99_ms"]
        # a loaded point: arrivals faster than single batches are served, 1e5 frequencies
        st2 = synth.stream(seed=5100, n_obj=max(2000, args.serve_objects // 5), rate_hz=60_000.0,
                           n_freq=100_000)
        rep2, _ = serve.replay(st2, slots=3, max_batch=4096, hbm_budget_bytes=4 << 30)
        rep2["workload"] = (f"{st2.size.size} objects, Poisson 60000 objects/s, sizes "
                            "round(LogNormal(ln 80, 0.8)) in [10, 1000], 1e5 frequencies")
        extra["serving_loaded"] = rep2

    # the CPU baseline, and the side legs above, at one GPU only (under torchrun the other
    # GPUs would wait on them)
    cpu = cpu_baseline(w, args.cpu_freqs) if args.cpu_freqs and world == 1 else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("f32 via split-f16 tensor MMAs (FP64 phase anchors)" if tensor_form
                      else "f32 (FP64 phase anchors)"),
            "data": "synthetic (seeded log-normal batch, stands in for the reference's missing "
                    "999-object file)",
            "config": {"workload": "lognormal_999obj_1e6freq_standard", "n_obj": w.n_obj,
                       "rows": w.n_rows, "n_freq": w.n_freq, "seed": w.seed,
                       "form": "mixed, tensor-core" if tensor_form else "mixed, CUDA-core",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "fmin": w.fmin, "fmax": w.fmax},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches, **extra}
    print(json.dumps(line), flush=True)
    eng.close()


if __name__ == "__main__":
    main()
