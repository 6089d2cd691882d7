"""TEST INFRASTRUCTURE ONLY: ctypes binding of the C oracle (oracle/ls_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs
import this module. It restates the reference's CPU path (source/main.cu modes 4/5)
in FP64; see ls_oracle.c for the line-by-line citations.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblsoracle.so"

_lib = None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    src = HERE / "ls_oracle.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        LIB.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-fopenmp",
                        "-ffp-contract=off", "-fvisibility=hidden", str(src), "-o", str(LIB), "-lm"],
                       check=True)
    lib = ctypes.CDLL(str(LIB))
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
    lib.lso_batch_pgram.argtypes = [ctypes.c_int, dp, dp, dp, up, up, ctypes.c_uint32,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                    ctypes.c_uint32, ctypes.c_int, dp, ctypes.c_int]
    lib.lso_batch_pgram.restype = ctypes.c_int
    lib.lso_std_power.argtypes = [dp, dp, ctypes.c_uint32, ctypes.c_double]
    lib.lso_std_power.restype = ctypes.c_double
    lib.lso_gen_power.argtypes = [dp, dp, dp, ctypes.c_uint32, ctypes.c_double]
    lib.lso_gen_power.restype = ctypes.c_double
    lib.lso_precenter.argtypes = [dp, dp, ctypes.c_uint32]
    lib.lso_norm_factor.argtypes = [dp, ctypes.c_uint32]
    lib.lso_norm_factor.restype = ctypes.c_double
    lib.lso_object_ranges.argtypes = [up, ctypes.c_uint32, up, up, ctypes.c_uint32]
    lib.lso_object_ranges.restype = ctypes.c_uint32
    lib.lso_omega.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_uint32]
    lib.lso_omega.restype = ctypes.c_double
    lib.lso_argmax.argtypes = [dp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                               ctypes.POINTER(ctypes.c_double)]
    lib.lso_top3.argtypes = [dp, ctypes.c_uint32, up, dp]
    lib.lso_max_threads.restype = ctypes.c_int
    _lib = lib
    return lib


def max_threads() -> int:
    return int(_load().lso_max_threads())


def object_ranges(obj_id):
    """(idx_min, idx_max) inclusive, source/main.cu:468-510."""
    ids = np.ascontiguousarray(obj_id, dtype=np.uint32)
    lib = _load()
    n = ids.size
    lo = np.zeros(max(n, 1), np.uint32)
    hi = np.zeros(max(n, 1), np.uint32)
    k = lib.lso_object_ranges(ids, n, lo, hi, max(n, 1))
    return lo[:k].copy(), hi[:k].copy()


def batch_pgram(variant, t, y, dy, offsets, fmin, df, n_freq=None, kidx=None, normalize=True,
                nthreads=0):
    """Periodogram [n_obj, nk] on grid indices kidx (default 0..n_freq-1), FP64.

    variant 0 standard (normalized by 2/(N var) when normalize), 1 generalized (y is
    pre-centered first, as the reference does; the input array is not modified).
    Returns (pgram, y_after) where y_after is the pre-centered copy of y.
    """
    lib = _load()
    t = np.ascontiguousarray(t, dtype=np.float64)
    y2 = np.array(y, dtype=np.float64, copy=True)
    dy = np.ascontiguousarray(np.ones_like(t) if dy is None else dy, dtype=np.float64)
    offs = np.asarray(offsets, dtype=np.int64)
    lo = np.ascontiguousarray(offs[:-1], dtype=np.uint32)
    hi = np.ascontiguousarray(offs[1:] - 1, dtype=np.uint32)
    if kidx is None:
        nk = int(n_freq)
        kp = None
    else:
        kidx = np.ascontiguousarray(kidx, dtype=np.uint32)
        nk = kidx.size
        kp = kidx.ctypes.data_as(ctypes.c_void_p)
    out = np.zeros(lo.size * nk, np.float64)
    rc = lib.lso_batch_pgram(int(variant), t, y2, dy, lo, hi, lo.size, float(fmin), float(df), kp,
                             nk, int(bool(normalize)), out, int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle failed: {rc}")
    return out.reshape(lo.size, nk), y2


def argmax(p):
    """(index, power) with the reference's first-maximum rule (source/main.cu:1545-1563)."""
    lib = _load()
    p = np.ascontiguousarray(p, dtype=np.float64)
    i = ctypes.c_uint32()
    v = ctypes.c_double()
    lib.lso_argmax(p, p.size, ctypes.byref(i), ctypes.byref(v))
    return int(i.value), float(v.value)


def top3(p):
    """The three best (index, power) pairs, best first, by the reference's three scans
    (source/main.cu:1165-1219): arrays (idx[3], power[3])."""
    lib = _load()
    p = np.ascontiguousarray(p, dtype=np.float64)
    idx = np.zeros(3, np.uint32)
    pw = np.zeros(3, np.float64)
    lib.lso_top3(p, p.size, idx, pw)
    return idx, pw


def float_grid(min_freq: float, max_freq: float, n_freq: int):
    """(fmin, df) of the float builds' GPU grid: the limits rounded to float, the step
    computed in double and held in float (source/kernel.cu:517 with DTYPE=float)."""
    f0 = float(np.float32(min_freq))
    f1 = float(np.float32(max_freq))
    return f0, float(np.float32((f1 - f0) / (n_freq * 1.0)))
