"""Generate the golden fixtures in tests/golden/ from the reference's own CPU path.

Run where the reference checkout is present (LSGB_REFERENCE_DIR, default /root/reference)
and its CPU libraries are built by ``make -C oracle ref`` (oracle/_ref/libpyls*.so):

    python tests/golden/make_golden.py

Every fixture holds the inputs and the reference's outputs of LombScarglePy in
CPU mode 5 (one object) or 4 (batch), double and float builds. Inputs are the
reference's test objects (data/8205_normalized*.txt: the 3,555-observation
synthetic object of the paper; data/243_normalized_ztf_filter2.txt: 29 ZTF
observations) and small seeded batches from gpu_lomb_scargle_gb300.synth.
The fixtures let the tests pin the oracle and the engine without the reference.
"""
from __future__ import annotations

import ctypes
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from gpu_lomb_scargle_gb300 import synth  # noqa: E402

REF = Path(os.environ.get("LSGB_REFERENCE_DIR", "/root/reference"))
REF_LIB = ROOT / "oracle" / "_ref"
OUT = Path(__file__).resolve().parent
TWO_PI = 2.0 * np.pi


def ref_call(error: bool, dtype: str, obj_id, t, y, dy, fmin, fmax, nf, mode):
    """LombScarglePy of the reference build; returns (pgram, y after the call)."""
    lib = ctypes.CDLL(str(REF_LIB / ("libpyls%s%s.so" % ("error" if error else "noerror", dtype))))
    npdt = np.float32 if dtype == "float" else np.float64
    arr = np.ctypeslib.ndpointer(dtype=npdt, flags="C_CONTIGUOUS")
    uarr = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
    lib.LombScarglePy.argtypes = [uarr, arr, arr, arr, ctypes.c_uint, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_uint, ctypes.c_int, arr]
    ids = np.ascontiguousarray(obj_id, np.uint32)
    tt = np.ascontiguousarray(t, npdt)
    yy = np.array(y, dtype=npdt, copy=True)
    dd = np.ascontiguousarray(dy, npdt)
    nobj = 1 if mode in (2, 5) else int(np.count_nonzero(np.diff(ids)) + 1)
    pg = np.zeros(nobj * nf, npdt)
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp())  # the reference appends gpu_stats.txt to the working directory
    try:
        lib.LombScarglePy(ids, tt, yy, dd, len(tt), fmin, fmax, nf, mode, pg)
    finally:
        os.chdir(cwd)
    return pg.reshape(nobj, nf), yy


def load_ref_data(name, error):
    d = np.loadtxt(REF / "data" / name, delimiter=",")
    dy = d[:, 3].copy() if error else np.ones(len(d))
    return d[:, 0].astype(np.uint32), d[:, 1].copy(), d[:, 2].copy(), dy


def main():
    if not (REF_LIB / "libpylsnoerrordouble.so").exists():
        raise SystemExit("build the reference CPU libraries first: make -C oracle ref")
    fx = {}
    # --- 8205, standard and generalized, ordinary 0.1..10 -> angular, 8000 frequencies
    lo, hi, nf = TWO_PI * 0.1, TWO_PI * 10.0, 8000
    for err, name in ((False, "8205_normalized.txt"), (True, "8205_normalized_with_error.txt")):
        ids, t, y, dy = load_ref_data(name, err)
        tag = "8205_%s" % ("gen" if err else "std")
        fx[tag + "_t"], fx[tag + "_y"], fx[tag + "_dy"] = t, y, dy
        for dt in ("double", "float"):
            pg, ya = ref_call(err, dt, ids, t, y, dy, lo, hi, nf, 5)
            fx[f"{tag}_{dt}_pgram"] = pg[0]
            fx[f"{tag}_{dt}_yafter"] = ya
    fx["8205_grid"] = np.array([lo, hi, nf], np.float64)

    # --- 243 (JD times ~2.4587e6), standard, CLI parameters of README.md:82-96
    ids, t, y, dy = load_ref_data("243_normalized_ztf_filter2.txt", False)
    fx["243_t"], fx["243_y"] = t, y
    pg, _ = ref_call(False, "double", ids, t, y, dy, 3.142, 150.796, 1_000_000, 5)
    fx["243_1e6_argmax"] = np.array([np.argmax(pg[0]), pg[0].max()])
    fx["243_1e6_window"] = pg[0][max(0, np.argmax(pg[0]) - 2000): np.argmax(pg[0]) + 2000]
    fx["243_1e6_window_start"] = np.array([max(0, np.argmax(pg[0]) - 2000)])
    pg, _ = ref_call(False, "double", ids, t, y, dy, 3.142, 150.796, 5000, 5)
    fx["243_5000_pgram"] = pg[0]

    # --- 8205 with error, CLI parameters of README.md:121-136 (1e6 frequencies)
    ids, t, y, dy = load_ref_data("8205_normalized_with_error.txt", True)
    pg, _ = ref_call(True, "double", ids, t, y, dy, 3.14159, 150.79645, 1_000_000, 5)
    k = int(np.argmax(pg[0]))
    fx["8205_gen_1e6_argmax"] = np.array([k, pg[0][k]])
    fx["8205_gen_1e6_window"] = pg[0][k - 1000: k + 1000]
    fx["8205_gen_1e6_window_start"] = np.array([k - 1000])

    # --- seeded batches (12 objects), mode 4, double and float builds
    for err in (False, True):
        w = synth.lognormal_batch(seed=777 + err, n_obj=12, n_freq=1500, error=err)
        tag = "batch_%s" % ("gen" if err else "std")
        fx[tag + "_ids"], fx[tag + "_t"], fx[tag + "_y"], fx[tag + "_dy"] = w.obj_id, w.t, w.y, w.dy
        fx[tag + "_grid"] = np.array([w.fmin, w.fmax, w.n_freq], np.float64)
        for dt in ("double", "float"):
            pg, ya = ref_call(err, dt, w.obj_id, w.t, w.y, w.dy, w.fmin, w.fmax, w.n_freq, 4)
            fx[f"{tag}_{dt}_pgram"] = pg
            fx[f"{tag}_{dt}_yafter"] = ya
    np.savez_compressed(OUT / "ref_cpu_golden.npz", **fx)
    print("wrote", OUT / "ref_cpu_golden.npz", sum(v.nbytes for v in fx.values()) / 1e6, "MB raw")


if __name__ == "__main__":
    main()
