"""Failure paths, made on the host or by a wait that is given no time; nothing here faults
or hangs a GPU.

* Invalid arguments are refused before any launch (LSGB_ERR_INVALID): no objects, an
  empty object, offsets that decrease, a missing dy for the generalized variant.
* Invalid data -- a non-finite time or magnitude, a non-finite or non-positive dy for the
  generalized variant -- has no defined periodogram (the reference computes NaN or infinite
  powers from it). The statistics kernel flags it; host calls return LSGB_ERR_INVALID,
  device calls and plans report LSGB_STATUS_BAD_INPUT, the serving loop stops with an error.
* A bounded pipeline wait of the tensor-form kernel that runs out (here: a wait limit of one
  cycle) aborts the launch: every role leaves its loop, the issued copies and MMAs are waited
  for, TMEM is freed, and the call reports the timeout. The next call on the same engine
  must be correct again.
The reference has no counterpart: it exits the process on a CUDA error
(source/main.cu:38-46) and never checks its inputs.
"""
import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import engine as E
from gpu_lomb_scargle_gb300 import synth
from gpu_lomb_scargle_gb300.engine import LsgbError
from oracle import pyoracle
from tests.gpu_helpers import MIXED_ATOL, check_best, mixed_abs_err

pytestmark = pytest.mark.gpu
ERR_INVALID, ERR_CUDA = -1, -2


@pytest.fixture(scope="module")
def eng(native_libs, cuda_ok):
    e = E.Engine(0)
    yield e
    e.close()


def batch(seed=3, n_obj=20, n_freq=6000, error=False):
    return synth.lognormal_batch(seed=seed, n_obj=n_obj, n_freq=n_freq, error=error)


def check_correct(eng, w, precision="mixed"):
    r = eng.run_host(0, precision, w.t, w.y, None, w.offsets, w.fmin, w.df, w.n_freq,
                     want_pgram=True)
    ref, _ = pyoracle.batch_pgram(0, w.t, w.y, None, w.offsets, w.fmin, w.df, n_freq=w.n_freq)
    assert mixed_abs_err(r.pgram, ref) < MIXED_ATOL
    assert check_best(r.best_idx, ref, tol=MIXED_ATOL) == []


@pytest.mark.parametrize("offsets,why", [
    (np.array([0], np.uint64), "no objects"),
    (np.array([0, 10, 10, 20], np.uint64), "an empty object"),
    (np.array([0, 15, 12, 20], np.uint64), "decreasing offsets"),
    (np.array([1, 10, 20], np.uint64), "offsets[0] != 0"),
])
def test_invalid_layout_refused(eng, offsets, why):
    w = batch(n_obj=2)
    with pytest.raises(LsgbError) as ei:
        eng.run_host(0, "mixed", w.t[:20], w.y[:20], None, offsets, w.fmin, w.df, 100)
    assert ei.value.status == ERR_INVALID, why


def test_generalized_without_dy_refused(eng):
    w = batch(n_obj=2, error=True)
    with pytest.raises(LsgbError) as ei:
        eng.run_host(1, "plain", w.t, w.y, None, w.offsets, w.fmin, w.df, 100)
    assert ei.value.status == ERR_INVALID


def test_zero_frequencies_give_the_reference_start(eng):
    """No frequency: nothing is computed and every object reports (index 0, power 0), the
    start value of the reference's argmax (source/main.cu:1545-1563)."""
    w = batch(n_obj=4)
    r = eng.run_host(0, "mixed", w.t, w.y, None, w.offsets, w.fmin, w.df, 0)
    np.testing.assert_array_equal(r.best_idx, 0)
    np.testing.assert_array_equal(r.best_power, 0)


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("what", ["nan_t", "inf_y", "zero_dy", "negative_dy", "nan_dy"])
def test_invalid_data_reported(eng, precision, what):
    variant = 1 if what.endswith("dy") else 0
    w = batch(n_obj=8, error=bool(variant))
    t, y, dy = w.t.copy(), w.y.copy(), w.dy.copy()
    row = int(w.offsets[5]) + 3  # inside object 5
    if what == "nan_t":
        t[row] = np.nan
    elif what == "inf_y":
        y[row] = np.inf
    elif what == "zero_dy":
        dy[row] = 0.0
    elif what == "negative_dy":
        dy[row] = -0.05
    else:
        dy[row] = np.nan
    with pytest.raises(LsgbError) as ei:
        eng.run_host(variant, precision, t, y, dy if variant else None, w.offsets, w.fmin, w.df,
                     w.n_freq, normalize=(variant == 0))
    assert ei.value.status == ERR_INVALID and "invalid input" in str(ei.value)
    # the word was cleared: the next call with good data succeeds and is right
    check_correct(eng, batch(seed=4))


def test_invalid_data_on_the_device_path_and_in_plans(eng):
    import torch
    w = batch(n_obj=6)
    dev = torch.device("cuda:0")
    t = torch.tensor(w.t, device=dev)
    y = torch.tensor(w.y, device=dev)
    t[int(w.offsets[2])] = float("nan")
    bi = torch.zeros(w.n_obj, dtype=torch.int32, device=dev)
    eng.run_device(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, best_idx=bi)
    assert eng.status() == E.STATUS_BAD_INPUT
    assert eng.status() == 0  # read and reset
    plan = eng.plan(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, best_idx=bi)
    plan.launch()
    with pytest.raises(LsgbError) as ei:
        plan.info(kernel_time=True)
    assert ei.value.status == ERR_INVALID
    t[int(w.offsets[2])] = float(w.t[int(w.offsets[2])])  # repaired in place
    plan.launch()
    assert plan.info(kernel_time=True)[2] > 0.0
    plan.close()


def test_lombscarglepy_reports_invalid_data(native_libs, cuda_ok):
    from gpu_lomb_scargle_gb300 import lombscarglegpu as lsg
    lib = lsg._library(False, "double")
    w = batch(n_obj=3)
    t = w.t.copy()
    t[1] = np.nan
    pg = np.zeros(3 * 500)
    lib.LombScarglePy(np.ascontiguousarray(w.obj_id, np.uint32), t, w.y.copy(), np.ones_like(t),
                      t.size, 1.0, 20.0, 500, 1, pg)
    assert lib.LombScarglePy_last_status() == ERR_INVALID


def test_serving_loop_stops_on_invalid_data(native_libs, cuda_ok):
    from gpu_lomb_scargle_gb300.serve import Server
    srv = Server(n_freq=3000, fmin=1.0, df=0.01, slots=1)
    try:
        w = batch(n_obj=1)
        y = w.y.copy()
        y[0] = np.nan
        srv.submit(7, w.t, y)
        failed = None
        for _ in range(400):
            try:
                srv.poll()
            except LsgbError as e:
                failed = e
                break
            import time
            time.sleep(0.005)
        assert failed is not None and "non-finite" in str(failed)
    finally:
        srv.close()


@pytest.mark.parametrize("variant", [0, 1])
def test_pipeline_wait_timeout_is_reported_and_recovered(native_libs, cuda_ok, variant):
    """A wait limit of one cycle makes the tensor kernel's first wait that is not already
    complete run out: the launch aborts cleanly and the call reports the timeout; with the
    default limit back, the same engine gives correct results (its TMEM was freed and its
    status word cleared)."""
    e = E.Engine(0)
    try:
        w = batch(seed=11 + variant, n_obj=30, error=bool(variant))
        y = w.y
        if variant:
            _, y = pyoracle.batch_pgram(1, w.t, w.y, w.dy, w.offsets, w.fmin, w.df, n_freq=1)
        e.set_wait_limit(1)
        with pytest.raises(LsgbError) as ei:
            e.run_host(variant, "mixed", w.t, y, w.dy if variant else None, w.offsets, w.fmin,
                       w.df, w.n_freq, normalize=(variant == 0))
        assert ei.value.status == ERR_CUDA and "timed out" in str(ei.value)
        e.set_wait_limit(0)
        r = e.run_host(variant, "mixed", w.t, y, w.dy if variant else None, w.offsets, w.fmin,
                       w.df, w.n_freq, normalize=(variant == 0), want_pgram=True)
        ref, _ = pyoracle.batch_pgram(variant, w.t, y, w.dy, w.offsets, w.fmin, w.df,
                                      n_freq=w.n_freq, normalize=(variant == 0))
        assert mixed_abs_err(r.pgram, ref) < MIXED_ATOL
        assert check_best(r.best_idx, ref, tol=MIXED_ATOL) == []
    finally:
        e.close()


def test_timeout_on_the_device_path_is_in_the_status(native_libs, cuda_ok):
    import torch
    e = E.Engine(0)
    try:
        w = batch(seed=21, n_obj=12)
        dev = torch.device("cuda:0")
        t = torch.tensor(w.t, device=dev)
        y = torch.tensor(w.y, device=dev)
        bi = torch.zeros(w.n_obj, dtype=torch.int32, device=dev)
        e.set_wait_limit(1)
        e.run_device(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, best_idx=bi)
        assert e.status() & E.STATUS_TIMEOUT
        e.set_wait_limit(0)
        e.run_device(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, best_idx=bi)
        assert e.status() == 0
    finally:
        e.close()
