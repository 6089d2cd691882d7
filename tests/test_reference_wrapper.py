"""The reference's own Python wrapper (source/lombscarglegpu.py), loaded unchanged from the
reference checkout, driving these libraries through ctypes exactly as it drives its own:
it loads libpyls{noerror,error}{float,double}.so from the working directory
(source/lombscarglegpu.py:279-287) and calls LombScarglePy.

Two things in that file predate NumPy 2 and need help from the caller, not from the
libraries: np.asfarray (used at :183 and :296-299) was removed in NumPy 2.0, so the test
puts an equivalent back for the duration of the call; and its check `magDY==None` (:259)
compares an ndarray elementwise, so in error mode magDY is passed as a list.

The reference checkout is found through LSGB_REFERENCE_DIR (default: where this container
mounts it); machines without it skip these tests.
"""
import contextlib
import importlib.util
import os
from pathlib import Path

import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import _native
from tests.gpu_helpers import PLAIN_RTOL, plain_rel_err

REF_DIR = Path(os.environ.get("LSGB_REFERENCE_DIR", "/root/reference"))
WRAPPER = REF_DIR / "source" / "lombscarglegpu.py"
TWO_PI = 2.0 * np.pi


@pytest.fixture(scope="module")
def ref_wrapper(native_libs):
    if not WRAPPER.exists():
        pytest.skip("the reference checkout is not present")
    spec = importlib.util.spec_from_file_location("reference_lombscarglegpu", WRAPPER)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@contextlib.contextmanager
def numpy1_and_libdir():
    """np.asfarray as NumPy 1 had it, and the libraries' directory as the working directory
    (where the wrapper looks for them)."""
    had = hasattr(np, "asfarray")
    if not had:
        np.asfarray = lambda a, dtype=float: np.asarray(a, dtype=dtype)
    cwd = os.getcwd()
    os.chdir(_native.LIB_DIR)
    try:
        yield
    finally:
        os.chdir(cwd)
        if not had:
            del np.asfarray


@pytest.mark.parametrize("error", [False, True])
def test_reference_wrapper_cpu_single_object(ref_wrapper, golden, error):
    tag = "8205_gen" if error else "8205_std"
    lo, hi, nf = golden["8205_grid"]  # angular; the wrapper takes ordinary frequencies
    t, y, dy = golden[tag + "_t"], golden[tag + "_y"], golden[tag + "_dy"]
    with numpy1_and_libdir():
        ids, periods, pgram = ref_wrapper.lombscargle(
            np.zeros(t.size, int), t, y.copy(), lo / TWO_PI, hi / TWO_PI, error, "CPU",
            magDY=list(dy) if error else None, freqToTest=int(nf), dtype="double")
    ref = golden[tag + "_double_pgram"]
    assert pgram.shape == (1, int(nf))
    assert plain_rel_err(pgram[0], ref) < PLAIN_RTOL
    k = int(np.argmax(ref))
    assert abs(periods[0] - 1.0 / (lo / TWO_PI + k * (hi - lo) / TWO_PI / nf)) < 1e-12


def test_reference_wrapper_cpu_batch(ref_wrapper, golden):
    lo, hi, nf = golden["batch_std_grid"]
    with numpy1_and_libdir():
        ids, periods, pgram = ref_wrapper.lombscargle(
            golden["batch_std_ids"], golden["batch_std_t"], golden["batch_std_y"].copy(),
            lo / TWO_PI, hi / TWO_PI, False, "CPU", freqToTest=int(nf), dtype="double")
    assert pgram.shape == golden["batch_std_double_pgram"].shape
    assert plain_rel_err(pgram, golden["batch_std_double_pgram"]) < PLAIN_RTOL
    assert list(ids) == sorted(set(golden["batch_std_ids"].tolist()))
