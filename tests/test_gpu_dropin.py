"""The drop-in libraries' GPU modes (MODE 1 batch, MODE 2 single object) through
LombScarglePy, against the reference's own CPU build (golden fixtures) and the oracle.

Double builds (plain FP64 form): <= 1e-9 relative. Float builds (mixed form on float
inputs): <= 1e-4 absolute against the FP64 oracle evaluated on the same float-rounded
inputs and the float build's frequency grid; the reference's own float build is looser
than that, so it is compared only through the best periods of its published examples.
"""
import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import lombscarglegpu as lsg
from oracle import pyoracle
from tests.gpu_helpers import MIXED_ATOL, PLAIN_RTOL, check_best, mixed_abs_err, plain_rel_err

pytestmark = pytest.mark.gpu
TWO_PI = 2.0 * np.pi


def call(err, dtype, ids, t, y, dy, fmin, fmax, nf, mode):
    lib = lsg._library(err, dtype)
    npdt = np.float32 if dtype == "float" else np.float64
    nobj = 1 if mode in (2, 5) else int(np.count_nonzero(np.diff(ids)) + 1)
    pg = np.zeros(nobj * nf, npdt)
    yy = np.array(y, npdt)
    lib.LombScarglePy(np.ascontiguousarray(ids, np.uint32), np.ascontiguousarray(t, npdt), yy,
                      np.ascontiguousarray(dy, npdt), len(t), fmin, fmax, nf, mode, pg)
    assert lib.LombScarglePy_last_status() == 0
    return pg.reshape(nobj, nf), yy


@pytest.mark.parametrize("err", [False, True])
def test_double_builds_mode2_match_reference_cpu(native_libs, cuda_ok, golden, err):
    tag = "8205_gen" if err else "8205_std"
    lo, hi, nf = golden["8205_grid"]
    t, y, dy = golden[tag + "_t"], golden[tag + "_y"], golden[tag + "_dy"]
    pg, ya = call(err, "double", np.zeros(t.size), t, y, dy, lo, hi, int(nf), 2)
    ref = golden[tag + "_double_pgram"]
    assert plain_rel_err(pg[0], ref) < PLAIN_RTOL
    assert np.argmax(pg[0]) == np.argmax(ref)
    # the generalized build pre-centers the caller's magY in place, as the reference does
    np.testing.assert_allclose(ya, golden[tag + "_double_yafter"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("err", [False, True])
def test_double_builds_mode1_match_reference_cpu(native_libs, cuda_ok, golden, err):
    tag = "batch_gen" if err else "batch_std"
    lo, hi, nf = golden[tag + "_grid"]
    pg, ya = call(err, "double", golden[tag + "_ids"], golden[tag + "_t"], golden[tag + "_y"],
                  golden[tag + "_dy"], lo, hi, int(nf), 1)
    ref = golden[tag + "_double_pgram"]
    assert plain_rel_err(pg, ref) < PLAIN_RTOL
    assert check_best(np.argmax(pg, axis=1), ref) == []
    np.testing.assert_allclose(ya, golden[tag + "_double_yafter"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("err", [False, True])
@pytest.mark.parametrize("mode", [1, 2])
def test_float_builds_against_oracle(native_libs, cuda_ok, golden, err, mode):
    tag = ("batch_" if mode == 1 else "8205_") + ("gen" if err else "std")
    if mode == 1:
        lo, hi, nf = golden[tag + "_grid"]
        ids = golden[tag + "_ids"]
    else:
        lo, hi, nf = golden["8205_grid"]
        ids = np.zeros(golden[tag + "_t"].size)
    nf = int(nf)
    t32 = golden[tag + "_t"].astype(np.float32)
    y32 = golden[tag + "_y"].astype(np.float32)
    dy32 = golden[tag + "_dy"].astype(np.float32)
    pg, ya = call(err, "float", ids, t32, y32, dy32, lo, hi, nf, mode)
    assert pg.dtype == np.float32
    fmin, df = pyoracle.float_grid(lo, hi, nf)
    offs = (np.concatenate([[0], np.nonzero(np.diff(ids))[0] + 1, [ids.size]]) if mode == 1
            else np.array([0, ids.size]))
    # the oracle on the same float inputs (the library's pre-centered magY for err)
    y_in = ya.astype(np.float64) if err else y32.astype(np.float64)
    ref, _ = pyoracle.batch_pgram(1 if err else 0, t32.astype(np.float64), y_in,
                                  dy32.astype(np.float64), offs, fmin, df, n_freq=nf)
    assert mixed_abs_err(pg, ref) < MIXED_ATOL
    assert check_best(np.argmax(pg, axis=1), ref, tol=MIXED_ATOL) == []


@pytest.mark.parametrize("error,period", [(True, 0.564739), (False, 0.564729)])
def test_mirror_api_reproduces_published_python_example(native_libs, cuda_ok, golden, error,
                                                        period):
    """python_output_lomb_scargle_test_example.txt:8 / :24: the float Python examples on
    the 8205 object (GPU mode, 330,000 frequencies over ordinary 0.1-10)."""
    tag = "8205_gen" if error else "8205_std"
    t, y, dy = golden[tag + "_t"], golden[tag + "_y"], golden[tag + "_dy"]
    ids, periods, pg = lsg.lombscargle(np.full(t.size, 8205), t, y, 0.1, 10.0, error, "GPU",
                                       magDY=dy if error else None, freqToTest=330_000,
                                       dtype="float")
    assert ids.tolist() == [8205] and pg.shape == (1, 330_000)
    assert round(float(periods[0]), 6) == period


def test_mirror_api_batch_gpu_double(native_libs, cuda_ok, golden):
    ids, t, y = golden["batch_std_ids"], golden["batch_std_t"], golden["batch_std_y"]
    lo, hi, nf = golden["batch_std_grid"]
    # the mirror takes ordinary frequencies and converts them to angular
    u, periods, pg = lsg.lombscargle(ids + 100, t, y, lo / TWO_PI, hi / TWO_PI, False, "GPU",
                                     freqToTest=int(nf), dtype="double")
    assert list(u) == sorted(set(ids + 100), key=list(ids + 100).index)
    assert plain_rel_err(pg, golden["batch_std_double_pgram"]) < PLAIN_RTOL
