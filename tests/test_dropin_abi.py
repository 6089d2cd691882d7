"""The drop-in libraries without a GPU: exported symbols, the CPU modes (MODE 4/5)
against the reference's own CPU build, and the failure path of the GPU modes."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import _native
from gpu_lomb_scargle_gb300 import lombscarglegpu as lsg

TWO_PI = 2.0 * np.pi


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def declared(header):
    """Function names declared in an include/*.h header."""
    import re
    txt = open(header).read()
    return set(re.findall(r"\b(lsgb_\w+|LombScarglePy\w*)\s*\(", txt))


def test_every_declared_symbol_is_exported(native_libs):
    root = _native.LIB_DIR.parents[1]
    lsgb_decl = declared(root / "include" / "lsgb.h")
    py_decl = declared(root / "include" / "lombscargle_py.h")
    assert lsgb_decl == set(_native.LSGB_SYMBOLS)  # the Python binding knows every entry point
    assert py_decl == set(_native.PYABI_SYMBOLS)
    syms = exported(_native.lib_path("liblsgb.so"))
    assert lsgb_decl <= syms, lsgb_decl - syms
    for lib in _native.DROPIN_LIBS:
        syms = exported(_native.lib_path(lib))
        assert py_decl <= syms, (lib, py_decl - syms)
        assert "LombScarglePy" in syms
        ctypes.CDLL(str(_native.lib_path(lib)))  # loads


def _call(lib_name, ids, t, y, dy, fmin, fmax, nf, mode, dtype):
    lib = lsg._library("error" in lib_name and "noerror" not in lib_name, dtype)
    npdt = np.float32 if dtype == "float" else np.float64
    nobj = 1 if mode in (2, 5) else int(np.count_nonzero(np.diff(ids)) + 1)
    pg = np.zeros(nobj * nf, npdt)
    yy = np.array(y, npdt)
    lib.LombScarglePy(np.ascontiguousarray(ids, np.uint32), np.ascontiguousarray(t, npdt), yy,
                      np.ascontiguousarray(dy, npdt), len(t), fmin, fmax, nf, mode, pg)
    return pg.reshape(nobj, nf), yy, lib.LombScarglePy_last_status()


@pytest.mark.parametrize("err", [False, True])
@pytest.mark.parametrize("dtype", ["double", "float"])
def test_cpu_mode5_matches_reference(native_libs, golden, err, dtype):
    tag = "8205_gen" if err else "8205_std"
    lo, hi, nf = golden["8205_grid"]
    name = "libpyls%s%s.so" % ("error" if err else "noerror", dtype)
    t, y, dy = golden[tag + "_t"], golden[tag + "_y"], golden[tag + "_dy"]
    pg, ya, st = _call(name, np.zeros(t.size, np.uint32), t, y, dy, lo, hi, int(nf), 5, dtype)
    assert st == 0
    ref = golden[f"{tag}_{dtype}_pgram"]
    if dtype == "double":
        np.testing.assert_allclose(pg[0], ref, rtol=1e-12, atol=0)
        np.testing.assert_allclose(ya, golden[f"{tag}_double_yafter"], rtol=0, atol=1e-13)
    else:
        # the reference's float pre-centering sums run in an OpenMP reduction order
        np.testing.assert_allclose(pg[0], ref, rtol=0, atol=2e-4 if err else 1e-6)
    assert np.argmax(pg[0]) == np.argmax(ref)


@pytest.mark.parametrize("err", [False, True])
@pytest.mark.parametrize("dtype", ["double", "float"])
def test_cpu_mode4_matches_reference(native_libs, golden, err, dtype):
    tag = "batch_gen" if err else "batch_std"
    lo, hi, nf = golden[tag + "_grid"]
    name = "libpyls%s%s.so" % ("error" if err else "noerror", dtype)
    pg, ya, st = _call(name, golden[tag + "_ids"], golden[tag + "_t"], golden[tag + "_y"],
                       golden[tag + "_dy"], lo, hi, int(nf), 4, dtype)
    assert st == 0
    ref = golden[f"{tag}_{dtype}_pgram"]
    if dtype == "double":
        np.testing.assert_allclose(pg, ref, rtol=1e-12, atol=0)
    else:
        np.testing.assert_allclose(pg, ref, rtol=0, atol=2e-4 if err else 1e-6)
    assert np.array_equal(np.argmax(pg, axis=1), np.argmax(ref, axis=1))


def test_unknown_mode_computes_nothing(native_libs):
    pg, _, st = _call("libpylsnoerrordouble.so", np.zeros(10, np.uint32), np.arange(10.0),
                      np.arange(10.0), np.ones(10), 1.0, 2.0, 5, 3, "double")
    assert st == 0 and not pg.any()


def test_gpu_mode_without_gpu_fails_loudly(native_libs):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; the failure path is for machines without one")
    pg, _, st = _call("libpylsnoerrordouble.so", np.zeros(10, np.uint32), np.arange(10.0),
                      np.sin(np.arange(10.0)), np.ones(10), 1.0, 2.0, 5, 2, "double")
    assert st == -4  # LSGB_ERR_NODEVICE: no silent CPU fallback
    assert not pg.any()


def test_mirror_api_cpu_mode(native_libs, golden):
    """lombscargle() of the mirrored reference API in CPU mode, one object."""
    t, y = golden["8205_std_t"], golden["8205_std_y"]
    ids, periods, pg = lsg.lombscargle(np.full(t.size, 8205), t, y, 0.1, 10.0, False, "CPU",
                                       freqToTest=8000, dtype="double")
    assert ids.tolist() == [8205]
    np.testing.assert_allclose(pg[0], golden["8205_std_double_pgram"], rtol=1e-12)
    k = int(np.argmax(pg[0]))
    assert periods[0] == 1.0 / (0.1 + (10.0 - 0.1) / 8000 * k)


def test_mirror_api_error_without_dmag_exits():
    with pytest.raises(SystemExit):
        lsg.lombscarglemain([0, 0, 0], [1.0, 2.0, 3.0], [1.0, 2.0, 1.0], 0.1, 1.0, True, "CPU",
                            freqToTest=4)


def test_auto_frequency_count():
    ids = np.repeat([0, 1], [5, 5])
    t = np.concatenate([np.linspace(0, 10, 5), np.linspace(3, 123, 5)])
    n = lsg.compute_num_freq_auto(ids, t, 0.1, 10.0)
    assert n == int((10.0 - 0.1) / (0.1 / 120.0))
