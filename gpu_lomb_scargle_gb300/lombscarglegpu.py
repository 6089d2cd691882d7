"""The reference's Python interface, bound to this repository's drop-in libraries.

``lombscargle`` has the signature, argument meaning and return value of
``lombscargle`` in source/lombscarglegpu.py:210-395:

    lombscargle(objId, timeX, magY, minFreq, maxFreq, error, mode, magDY=None,
                freqToTest="auto", dtype="float", verbose=False)
      -> (uniqueObjectIdsOrdered, periods, pgram[num_objects, freqToTest])

* ``minFreq``/``maxFreq`` are ordinary frequencies; they are converted to angular
  ones before the C call (:227-228) and ``maxFreq`` is exclusive.
* ``mode`` "GPU" or "CPU"; one object -> single-object mode (2 / 5), more -> batch
  mode (1 / 4) (:249-257).
* ``freqToTest="auto"`` picks N from the longest observing window (Richards et al.
  2011: df = 0.1 / window, :179-206).
* Object ids may be any values; objects are runs of equal ids, re-enumerated 0..K-1
  before the call (:270-271).
* ``periods`` are recomputed from ``argmax`` of each returned periodogram row in
  ordinary frequency (:381-383).
* ``error=True`` without ``magDY`` prints the reference's message and exits with
  status 0 (:261-263).

The shared libraries are loaded from this package's ``lib`` directory (the
reference loads them from the working directory, :279-287; copying the four
``libpyls*.so`` files there lets the reference's own wrapper use them unchanged).
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

from . import _native

__all__ = ["lombscargle", "lombscarglemain", "compute_num_freq_auto", "object_ranges"]


def object_ranges(obj_id):
    """(start, end inclusive, unique ids in order) of the runs of equal ids."""
    ids = np.asarray(obj_id)
    if ids.size == 0:
        return np.zeros(0, int), np.zeros(0, int), ids
    change = np.nonzero(ids[1:] != ids[:-1])[0] + 1
    start = np.concatenate([[0], change]).astype(int)
    end = np.concatenate([change - 1, [ids.size - 1]]).astype(int)
    return start, end, ids[start]


def compute_num_freq_auto(obj_id, time_x, fmin, fmax):
    """Number of frequencies from the longest observing window (source/lombscarglegpu.py:179-206)."""
    start, end, _ = object_ranges(obj_id)
    t = np.asarray(time_x, dtype=float)
    window = np.max(t[end] - t[start])
    delta_f = 0.1 / window
    n = int((fmax - fmin) / delta_f)
    print("*********************")
    print("Automatically generating the number of frequencies based on maximum observing window:")
    print("Max. Observing Window: %f, Delta f: %f" % (window, delta_f))
    print("Number of frequencies: ", n)
    print("*********************")
    return n


class _HiddenStdout:
    """Send file descriptor 1 to /dev/null for the duration (C printf output included)."""

    def __enter__(self):
        sys.stdout.flush()
        self._saved = os.dup(1)
        devnull = os.open(os.devnull, os.O_WRONLY)
        os.dup2(devnull, 1)
        os.close(devnull)
        return self

    def __exit__(self, *exc):
        sys.stdout.flush()
        os.dup2(self._saved, 1)
        os.close(self._saved)
        return False


def lombscargle(objId, timeX, magY, minFreq, maxFreq, error, mode, magDY=None, freqToTest="auto",
                dtype="float", verbose=False):
    if not verbose:
        with _HiddenStdout():
            return lombscarglemain(objId, timeX, magY, minFreq, maxFreq, error, mode, magDY,
                                   freqToTest, dtype)
    return lombscarglemain(objId, timeX, magY, minFreq, maxFreq, error, mode, magDY, freqToTest,
                           dtype, verbose)


def _library(error: bool, dtype: str) -> ctypes.CDLL:
    name = "libpyls%s%s.so" % ("error" if error else "noerror", dtype)
    lib = _native.load(name)
    ctype = ctypes.c_float if dtype == "float" else ctypes.c_double
    arr = np.ctypeslib.ndpointer(dtype=ctype, ndim=1, flags="CONTIGUOUS")
    uarr = np.ctypeslib.ndpointer(dtype=ctypes.c_uint, ndim=1, flags="CONTIGUOUS")
    lib.LombScarglePy.argtypes = [uarr, arr, arr, arr, ctypes.c_uint, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_uint, ctypes.c_int, arr]
    lib.LombScarglePy.restype = None
    lib.LombScarglePy_last_status.restype = ctypes.c_int
    return lib


def lombscarglemain(objId, timeX, magY, minFreq, maxFreq, error, mode, magDY=None,
                    freqToTest="auto", dtype="float", verbose=False):
    fmin_std, fmax_std = minFreq, maxFreq
    fmin_ang, fmax_ang = 2.0 * np.pi * minFreq, 2.0 * np.pi * maxFreq
    if isinstance(freqToTest, str) and freqToTest == "auto":
        freqToTest = compute_num_freq_auto(objId, timeX, fmin_std, fmax_std)
    n_obj_in = np.unique(np.asarray(objId)).size
    if mode == "GPU":
        setmode = 2 if n_obj_in == 1 else 1
    elif mode == "CPU":
        setmode = 5 if n_obj_in == 1 else 4
    else:
        raise ValueError("mode must be 'GPU' or 'CPU'")
    if error and magDY is None:
        print("[Python] Error: No input error array, but the error mode is True. Set error mode to False.")
        sys.exit(0)
    if dtype not in ("float", "double"):
        raise ValueError("dtype must be 'float' or 'double'")

    start, end, unique_ids = object_ranges(objId)
    enum_ids = np.repeat(np.arange(start.size), end - start + 1)
    size_data = enum_ids.size
    print("[Python] Number of rows in file: %d" % size_data)
    npdt = np.float32 if dtype == "float" else np.float64
    c_obj = np.ascontiguousarray(enum_ids, dtype=np.uint32)
    c_t = np.ascontiguousarray(np.asarray(timeX, dtype=float), dtype=npdt)
    c_y = np.ascontiguousarray(np.asarray(magY, dtype=float), dtype=npdt)
    dy = np.asarray(magDY, dtype=float) if error else np.full(size_data, 1.0)
    c_dy = np.ascontiguousarray(dy, dtype=npdt)
    n_obj = start.size
    print("[Python] Unique objects: %d" % n_obj)
    pgram = np.zeros(n_obj * int(freqToTest), dtype=npdt)
    print("[Python] Size of pgram in elems: %d (%f GiB)" % (pgram.size, pgram.nbytes / 2**30))
    lib = _library(bool(error), dtype)
    lib.LombScarglePy(c_obj, c_t, c_y, c_dy, ctypes.c_uint(size_data), ctypes.c_double(fmin_ang),
                      ctypes.c_double(fmax_ang), ctypes.c_uint(int(freqToTest)),
                      ctypes.c_int(setmode), pgram)
    status = lib.LombScarglePy_last_status()
    if status != 0:
        raise RuntimeError("LombScarglePy failed with lsgb status %d (see stderr)" % status)
    pgram = pgram.reshape(n_obj, int(freqToTest))
    df_std = (fmax_std - fmin_std) / int(freqToTest) * 1.0
    periods = 1.0 / (fmin_std + df_std * np.argmax(pgram, axis=1))
    if n_obj > 1:
        print("[Python] Sum of all periods: %f" % np.sum(periods))
    else:
        print("[Python] Period for object: %f" % periods[0])
    return unique_ids, periods, pgram
