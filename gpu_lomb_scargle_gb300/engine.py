"""Python binding of the engine's C ABI (include/lsgb.h).

``Engine.run_device`` takes CUDA tensors already resident in HBM (torch is used
only to own device memory and streams); ``Engine.run_host`` takes numpy arrays
and performs the copies inside the native call. Both compute on the GPU only.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native

STANDARD, GENERALIZED = 0, 1
STATUS_TIMEOUT, STATUS_BAD_INPUT = 1, 2
PLAIN_FP64, MIXED = 0, 1
F32, F64 = 0, 1

_PRECISIONS = {"plain": PLAIN_FP64, "plain_fp64": PLAIN_FP64, "mixed": MIXED}


class LsgbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"lsgb status {status}: {msg}")
        self.status = status


def _precision(p) -> int:
    return _PRECISIONS[p] if isinstance(p, str) else int(p)


def _dtype_code(dt) -> int:
    dt = np.dtype(dt)
    if dt == np.float32:
        return F32
    if dt == np.float64:
        return F64
    raise TypeError(f"unsupported dtype {dt}; use float32 or float64")


def offsets_from_ids(obj_id: np.ndarray) -> np.ndarray:
    """Row offsets of the contiguous runs of equal ids (source/main.cu:468-510)."""
    obj_id = np.asarray(obj_id)
    if obj_id.size == 0:
        return np.zeros(1, np.uint64)
    change = np.nonzero(obj_id[1:] != obj_id[:-1])[0] + 1
    return np.concatenate([[0], change, [obj_id.size]]).astype(np.uint64)


@dataclass
class Result:
    best_idx: np.ndarray
    best_power: np.ndarray
    pgram: np.ndarray | None


class Engine:
    """One engine per device. Not thread-safe: calls on one engine must be ordered."""

    def __init__(self, device: int = 0):
        self._lib = _native.lsgb()
        h = ctypes.c_void_p()
        rc = self._lib.lsgb_engine_create(int(device), ctypes.byref(h))
        self._check(rc)
        self._h = h
        self.device = device

    def _check(self, rc: int):
        if rc != 0:
            raise LsgbError(rc, self._lib.lsgb_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lsgb_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, variant: int, freqs_per_thread: int = 0, threads: int = 0,
                   min_ctas: int = 0, packed: int = -1, unroll: int = -1):
        self._check(self._lib.lsgb_set_tuning(self._h, variant, freqs_per_thread, threads,
                                              min_ctas, packed, unroll))

    def fp64_sincos_check(self, n: int = 1 << 22, scale: float = 1e3) -> float:
        """Largest |difference| of the plain form's FP64 sin/cos from CUDA's sincos()."""
        out = ctypes.c_double()
        self._check(self._lib.lsgb_fp64_sincos_check(self._h, int(n), float(scale),
                                                     ctypes.byref(out)))
        return float(out.value)

    def set_wait_limit(self, cycles: int):
        """Limit of the tensor form's bounded pipeline waits in SM cycles (0: default)."""
        self._check(self._lib.lsgb_set_wait_limit(self._h, int(cycles)))

    def status(self, stream=None) -> int:
        """LSGB_STATUS_* bits recorded by the device calls queued on `stream` so far (waits
        for the stream), and resets them."""
        import torch

        st = stream if stream is not None else torch.cuda.current_stream()
        out = ctypes.c_uint32(0)
        self._check(self._lib.lsgb_status_async(self._h, ctypes.byref(out),
                                                ctypes.c_void_p(st.cuda_stream)))
        st.synchronize()
        return int(out.value)

    def set_reanchor(self, interval: int):
        self._check(self._lib.lsgb_set_reanchor(self._h, int(interval)))

    def get_tuning(self, variant: int):
        out = (ctypes.c_int * 6)()
        self._check(self._lib.lsgb_get_tuning(self._h, variant, out))
        return tuple(out)[1:]

    def launch_info(self):
        k = ctypes.c_uint32()
        u = ctypes.c_uint64()
        self._check(self._lib.lsgb_last_launch_info(self._h, ctypes.byref(k), ctypes.byref(u)))
        return int(k.value), int(u.value)

    def last_kernel_ms(self) -> float:
        ms = ctypes.c_float()
        self._check(self._lib.lsgb_last_kernel_time(self._h, ctypes.byref(ms)))
        return float(ms.value)

    # ---- device-resident call -------------------------------------------------
    def run_device(self, variant, precision, t, y, dy, offsets, fmin, df, n_freq, normalize=True,
                   pgram=None, best_idx=None, best_power=None, stream=None):
        """t, y, dy, pgram, best_idx, best_power: CUDA tensors (or None); offsets: numpy uint64."""
        import torch

        if t.dtype == torch.float32:
            code = F32
        elif t.dtype == torch.float64:
            code = F64
        else:
            raise TypeError("t must be float32 or float64")
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        n_obj = offs.size - 1
        ptr = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None
        st = ctypes.c_void_p(stream.cuda_stream if stream is not None
                             else torch.cuda.current_stream().cuda_stream)
        rc = self._lib.lsgb_periodogram_device(
            self._h, int(variant), _precision(precision), code, ptr(t), ptr(y), ptr(dy),
            offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n_obj, float(fmin), float(df),
            int(n_freq), int(bool(normalize)), ptr(pgram), ptr(best_idx), ptr(best_power), st)
        self._check(rc)

    def plan(self, variant, precision, t, y, dy, offsets, fmin, df, n_freq, normalize=True,
             pgram=None, best_idx=None, best_power=None) -> "Plan":
        """A CUDA-graph plan of run_device with these (CUDA tensor) arguments."""
        return Plan(self, variant, precision, t, y, dy, offsets, fmin, df, n_freq, normalize,
                    pgram, best_idx, best_power)

    def run_device_top3(self, variant, precision, t, y, dy, offsets, fmin, df, n_freq,
                        normalize=True, pgram=None, top_idx=None, top_power=None, stream=None):
        """As run_device, with the three best frequencies per object: top_idx (int32/uint32)
        and top_power are CUDA tensors of n_obj x 3 (source/main.cu:1165-1219)."""
        import torch

        code = F32 if t.dtype == torch.float32 else F64
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        ptr = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None
        st = ctypes.c_void_p(stream.cuda_stream if stream is not None
                             else torch.cuda.current_stream().cuda_stream)
        self._check(self._lib.lsgb_periodogram_top3_device(
            self._h, int(variant), _precision(precision), code, ptr(t), ptr(y), ptr(dy),
            offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), offs.size - 1, float(fmin),
            float(df), int(n_freq), int(bool(normalize)), ptr(pgram), ptr(top_idx), ptr(top_power),
            st))

    # ---- host-buffer call -----------------------------------------------------
    def run_host(self, variant, precision, t, y, dy, offsets, fmin, df, n_freq, normalize=True,
                 want_pgram=False, out_pgram=None, out_idx=None, out_power=None) -> Result:
        t = np.ascontiguousarray(t)
        code = _dtype_code(t.dtype)
        y = np.ascontiguousarray(y, dtype=t.dtype)
        dy = None if dy is None else np.ascontiguousarray(dy, dtype=t.dtype)
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        n_obj = offs.size - 1
        pg = out_pgram
        if pg is None and want_pgram:
            pg = np.empty((n_obj, int(n_freq)), dtype=t.dtype)
        idx = out_idx if out_idx is not None else np.empty(n_obj, np.uint32)
        pw = out_power if out_power is not None else np.empty(n_obj, t.dtype)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
        rc = self._lib.lsgb_periodogram_host(
            self._h, int(variant), _precision(precision), code, vp(t), vp(y), vp(dy),
            offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n_obj, float(fmin), float(df),
            int(n_freq), int(bool(normalize)), vp(pg), vp(idx), vp(pw))
        self._check(rc)
        return Result(idx, pw, pg)

    def run_host_top3(self, variant, precision, t, y, dy, offsets, fmin, df, n_freq,
                      normalize=True, want_pgram=False) -> Result:
        """As run_host, with best_idx / best_power of shape (n_obj, 3): the three best
        frequencies of every object, best first (0 where fewer than three positive powers)."""
        t = np.ascontiguousarray(t)
        code = _dtype_code(t.dtype)
        y = np.ascontiguousarray(y, dtype=t.dtype)
        dy = None if dy is None else np.ascontiguousarray(dy, dtype=t.dtype)
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        n_obj = offs.size - 1
        pg = np.empty((n_obj, int(n_freq)), dtype=t.dtype) if want_pgram else None
        idx = np.empty((n_obj, 3), np.uint32)
        pw = np.empty((n_obj, 3), t.dtype)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
        self._check(self._lib.lsgb_periodogram_top3_host(
            self._h, int(variant), _precision(precision), code, vp(t), vp(y), vp(dy),
            offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n_obj, float(fmin), float(df),
            int(n_freq), int(bool(normalize)), vp(pg), vp(idx), vp(pw)))
        return Result(idx, pw, pg)


class Plan:
    """One batch shape captured in a CUDA graph (lsgb_plan_*); keeps its tensors alive."""

    def __init__(self, eng, variant, precision, t, y, dy, offsets, fmin, df, n_freq, normalize,
                 pgram, best_idx, best_power):
        import torch

        if t.dtype == torch.float32:
            code = F32
        elif t.dtype == torch.float64:
            code = F64
        else:
            raise TypeError("t must be float32 or float64")
        self._eng = eng
        self._keep = (t, y, dy, pgram, best_idx, best_power)
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        ptr = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None
        h = ctypes.c_void_p()
        eng._check(eng._lib.lsgb_plan_create(
            eng._h, int(variant), _precision(precision), code, ptr(t), ptr(y), ptr(dy),
            offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), offs.size - 1, float(fmin),
            float(df), int(n_freq), int(bool(normalize)), ptr(pgram), ptr(best_idx),
            ptr(best_power), ctypes.byref(h)))
        self._h = h

    def launch(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream()
        self._eng._check(self._eng._lib.lsgb_plan_launch(self._h, ctypes.c_void_p(st.cuda_stream)))

    def info(self, kernel_time=False):
        k = ctypes.c_uint32()
        u = ctypes.c_uint64()
        ms = ctypes.c_float()
        self._eng._check(self._eng._lib.lsgb_plan_info(self._h, ctypes.byref(k), ctypes.byref(u),
                                                       ctypes.byref(ms) if kernel_time else None))
        return int(k.value), int(u.value), (float(ms.value) if kernel_time else None)

    def close(self):
        if getattr(self, "_h", None):
            self._eng._lib.lsgb_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mixed_shapes():
    """Compiled mixed-kernel shapes: (variant, F, threads, min_ctas, packed, unroll)."""
    lib = _native.lsgb()
    n = lib.lsgb_mixed_shapes(None, 0)
    buf = (ctypes.c_int * (6 * n))()
    lib.lsgb_mixed_shapes(buf, n)
    return [tuple(buf[6 * i:6 * i + 6]) for i in range(n)]


_default: Engine | None = None


def default_engine() -> Engine:
    global _default
    if _default is None:
        _default = Engine(0)
    return _default
