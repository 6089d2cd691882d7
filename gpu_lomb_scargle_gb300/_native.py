"""Loading of the in-tree native libraries (built by ``gpu_lomb_scargle_gb300.build``).

There is no Python or CPU fallback: if a library is missing, loading raises
``NativeLibraryMissing`` with the build command to run.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "lib"

DROPIN_LIBS = ("libpylsnoerrorfloat.so", "libpylsnoerrordouble.so", "libpylserrorfloat.so",
               "libpylserrordouble.so")

# Symbols each library must export (the declarations of include/lsgb.h and
# include/lombscargle_py.h).
LSGB_SYMBOLS = ("lsgb_engine_create", "lsgb_engine_destroy", "lsgb_last_error", "lsgb_version",
                "lsgb_periodogram_device", "lsgb_periodogram_host", "lsgb_periodogram_top3_device",
                "lsgb_periodogram_top3_host", "lsgb_set_tuning",
                "lsgb_last_launch_info", "lsgb_last_kernel_time", "lsgb_mixed_shapes",
                "lsgb_get_tuning", "lsgb_periodogram_noalloc", "lsgb_server_create",
                "lsgb_server_submit", "lsgb_server_poll", "lsgb_server_stats", "lsgb_server_now",
                "lsgb_server_destroy", "lsgb_set_reanchor", "lsgb_fp64_sincos_check", "lsgb_plan_create",
                "lsgb_plan_launch", "lsgb_plan_info", "lsgb_plan_destroy", "lsgb_plan_status_async",
                "lsgb_status_async", "lsgb_set_wait_limit", "lsgb_server_peaks")
PYABI_SYMBOLS = ("LombScarglePy", "LombScarglePy_last_status")


class NativeLibraryMissing(RuntimeError):
    pass


_cache: dict[str, ctypes.CDLL] = {}


def lib_path(name: str) -> Path:
    return LIB_DIR / name


def load(name: str) -> ctypes.CDLL:
    if name in _cache:
        return _cache[name]
    p = lib_path(name)
    if not p.exists():
        raise NativeLibraryMissing(
            f"{p} is not built; run `python -m gpu_lomb_scargle_gb300.build` (CUDA 13, sm_103a)")
    lib = ctypes.CDLL(str(p))
    _cache[name] = lib
    return lib


def lsgb() -> ctypes.CDLL:
    lib = load("liblsgb.so")
    if not getattr(lib, "_lsgb_typed", False):
        c = ctypes
        vp, u32, u64p, dbl, i32 = c.c_void_p, c.c_uint32, c.POINTER(c.c_uint64), c.c_double, c.c_int
        lib.lsgb_engine_create.argtypes = [i32, c.POINTER(vp)]
        lib.lsgb_engine_create.restype = i32
        lib.lsgb_engine_destroy.argtypes = [vp]
        lib.lsgb_engine_destroy.restype = None
        lib.lsgb_last_error.restype = c.c_char_p
        lib.lsgb_version.restype = c.c_char_p
        common = [vp, i32, i32, i32, vp, vp, vp, u64p, u32, dbl, dbl, u32, i32, vp, vp, vp]
        lib.lsgb_periodogram_device.argtypes = common + [vp]
        lib.lsgb_periodogram_device.restype = i32
        lib.lsgb_periodogram_host.argtypes = common
        lib.lsgb_periodogram_host.restype = i32
        lib.lsgb_periodogram_top3_device.argtypes = common + [vp]
        lib.lsgb_periodogram_top3_device.restype = i32
        lib.lsgb_periodogram_top3_host.argtypes = common
        lib.lsgb_periodogram_top3_host.restype = i32
        lib.lsgb_set_tuning.argtypes = [vp, i32, i32, i32, i32, i32, i32]
        lib.lsgb_set_tuning.restype = i32
        lib.lsgb_last_launch_info.argtypes = [vp, c.POINTER(c.c_uint32), c.POINTER(c.c_uint64)]
        lib.lsgb_last_launch_info.restype = i32
        lib.lsgb_last_kernel_time.argtypes = [vp, c.POINTER(c.c_float)]
        lib.lsgb_last_kernel_time.restype = i32
        lib.lsgb_mixed_shapes.argtypes = [c.POINTER(c.c_int), i32]
        lib.lsgb_mixed_shapes.restype = i32
        lib.lsgb_get_tuning.argtypes = [vp, i32, c.POINTER(c.c_int)]
        lib.lsgb_get_tuning.restype = i32
        lib.lsgb_periodogram_noalloc.argtypes = [i32, i32, vp, vp, vp, u64p, u32, dbl, dbl, u32,
                                                 i32, vp, vp, vp, vp]
        lib.lsgb_periodogram_noalloc.restype = i32
        dp = c.POINTER(c.c_double)
        lib.lsgb_server_create.argtypes = [i32, i32, i32, dbl, dbl, u32, i32, u32, u32, c.c_uint64,
                                           c.POINTER(vp)]
        lib.lsgb_server_create.restype = i32
        lib.lsgb_server_submit.argtypes = [vp, c.c_uint64, dp, dp, dp, u32]
        lib.lsgb_server_submit.restype = i32
        lib.lsgb_server_poll.argtypes = [vp, u32, u64p, c.POINTER(c.c_uint32), dp, dp, dp]
        lib.lsgb_server_poll.restype = i32
        lib.lsgb_server_stats.argtypes = [vp, u64p]
        lib.lsgb_server_stats.restype = i32
        lib.lsgb_server_now.restype = dbl
        lib.lsgb_server_peaks.argtypes = [vp, u64p]
        lib.lsgb_server_peaks.restype = i32
        lib.lsgb_server_destroy.argtypes = [vp]
        lib.lsgb_server_destroy.restype = None
        lib.lsgb_set_reanchor.argtypes = [vp, u32]
        lib.lsgb_set_reanchor.restype = i32
        lib.lsgb_fp64_sincos_check.argtypes = [vp, u32, dbl, c.POINTER(c.c_double)]
        lib.lsgb_fp64_sincos_check.restype = i32
        lib.lsgb_plan_create.argtypes = common + [c.POINTER(vp)]
        lib.lsgb_plan_create.restype = i32
        lib.lsgb_plan_launch.argtypes = [vp, vp]
        lib.lsgb_plan_launch.restype = i32
        lib.lsgb_plan_info.argtypes = [vp, c.POINTER(c.c_uint32), c.POINTER(c.c_uint64),
                                       c.POINTER(c.c_float)]
        lib.lsgb_plan_info.restype = i32
        lib.lsgb_plan_destroy.argtypes = [vp]
        lib.lsgb_plan_destroy.restype = None
        lib.lsgb_plan_status_async.argtypes = [vp, c.POINTER(c.c_uint32), vp]
        lib.lsgb_plan_status_async.restype = i32
        lib.lsgb_status_async.argtypes = [vp, c.POINTER(c.c_uint32), vp]
        lib.lsgb_status_async.restype = i32
        lib.lsgb_set_wait_limit.argtypes = [vp, c.c_uint64]
        lib.lsgb_set_wait_limit.restype = i32
        lib._lsgb_typed = True
    return lib
