"""K-sliced units of the tensor form.

A batch with fewer (object, frequency tile) pairs than the GPU has SMs has every object's
observations cut into slices of at least 16 K-blocks (256 observations), summed on different
SMs; a finishing pass adds the slices' raw sums and forms the powers, the periodogram and the
best frequencies. These tests check that the split is taken (the launch's work units are a
multiple of the pairs) and that its results agree with the plain FP64 form on the same inputs
(the drop-in arithmetic, pinned to the oracle by the parity tests): powers within 1e-4
absolute, the best frequency and the top three identical or within a 1e-4 near-tie.
"""
import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import engine as E
from gpu_lomb_scargle_gb300 import synth
from oracle import pyoracle
from tests.gpu_helpers import MIXED_ATOL, check_best, mixed_abs_err

pytestmark = pytest.mark.gpu

TILE = {0: 8192, 1: 4096}  # frequencies per tensor-form unit (128 fine x 64 / 32 coarse steps)


@pytest.fixture(scope="module")
def eng(native_libs, cuda_ok):
    e = E.Engine(0)
    yield e
    e.close()


def _workload(kind, variant):
    rng = np.random.default_rng(7100 + variant)
    if kind == "single":
        w = synth.single_object(seed=7000 + variant, n_freq=100_000)
        offs = w.offsets
        t, y = w.t, w.y
    else:
        # three objects of 3,555, 1,000 and 600 observations: 223, 63 and 38 K-blocks, so
        # the shortest allows two slices
        parts = [synth.single_object(seed=7200 + i, n_obs=n, n_freq=10_000)
                 for i, n in enumerate((3555, 1000, 600))]
        t = np.concatenate([p.t for p in parts])
        y = np.concatenate([p.y for p in parts])
        offs = np.concatenate([[0], np.cumsum([p.t.size for p in parts])])
        w = parts[0]
    dy = rng.uniform(0.01, 0.1, t.size) if variant else None
    return t, y, dy, np.asarray(offs, np.uint64), w.fmin, w.df, w.n_freq


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("kind", ["single", "three"])
def test_sliced_units_match_plain_fp64(eng, variant, kind):
    t, y, dy, offs, fmin, df, nf = _workload(kind, variant)
    n_obj = offs.size - 1
    runs = {}
    for precision in ("plain", "mixed"):
        r = eng.run_host(variant, precision, t, y, dy, offs, fmin, df, nf,
                         normalize=(variant == 0), want_pgram=True)
        runs[precision] = r
        if precision == "mixed":
            _, units = eng.launch_info()
            pairs = n_obj * -(-nf // TILE[variant])
            assert units % pairs == 0 and units // pairs > 1, (units, pairs)
    ref = runs["plain"].pgram.reshape(n_obj, nf)
    got = runs["mixed"].pgram.reshape(n_obj, nf)
    assert mixed_abs_err(got, ref) < MIXED_ATOL
    assert not check_best(runs["mixed"].best_idx, ref, tol=MIXED_ATOL)
    # the best power is the periodogram's value at the best index
    rows = np.arange(n_obj)
    np.testing.assert_array_equal(runs["mixed"].best_power, got[rows, runs["mixed"].best_idx])


@pytest.mark.parametrize("variant", [0, 1])
def test_sliced_units_top3(eng, variant):
    t, y, dy, offs, fmin, df, nf = _workload("three", variant)
    n_obj = offs.size - 1
    ref = eng.run_host(variant, "plain", t, y, dy, offs, fmin, df, nf,
                       normalize=(variant == 0), want_pgram=True).pgram.reshape(n_obj, nf)
    r = eng.run_host_top3(variant, "mixed", t, y, dy, offs, fmin, df, nf,
                          normalize=(variant == 0), want_pgram=True)
    got = r.pgram.reshape(n_obj, nf)
    for o in range(n_obj):
        ridx, rpw = pyoracle.top3(ref[o])
        np.testing.assert_allclose(r.best_power[o], rpw, atol=MIXED_ATOL, rtol=0)
        for j in range(3):
            if r.best_idx[o, j] != ridx[j]:
                assert abs(ref[o, r.best_idx[o, j]] - rpw[j]) <= MIXED_ATOL, (o, j)
        # the three are the mixed periodogram's own three best, exactly
        gidx, gpw = pyoracle.top3(got[o])
        np.testing.assert_array_equal(r.best_idx[o], gidx)
        np.testing.assert_array_equal(r.best_power[o], gpw)


@pytest.mark.parametrize("n_freq", [1, 2, 7])
def test_sliced_units_with_few_frequencies(eng, n_freq):
    """One long object at 1, 2 and 7 frequencies: a single tile cut into many slices, the
    finishing pass covering only the first frequencies of its tile, and (at 1 and 2
    frequencies) a top three padded with (0, 0)."""
    w = synth.long_object(seed=7300, n_obs=5000, n_freq=n_freq)
    offs = np.asarray(w.offsets, np.uint64)
    ref = eng.run_host(0, "plain", w.t, w.y, None, offs, w.fmin, w.df, n_freq,
                       normalize=True, want_pgram=True).pgram.reshape(1, n_freq)
    r = eng.run_host(0, "mixed", w.t, w.y, None, offs, w.fmin, w.df, n_freq, normalize=True,
                     want_pgram=True)
    _, units = eng.launch_info()
    assert units > 1  # 5,000 observations = 313 K-blocks: sliced
    got = r.pgram.reshape(1, n_freq)
    assert mixed_abs_err(got, ref) < MIXED_ATOL
    assert not check_best(r.best_idx, ref, tol=MIXED_ATOL)
    t3 = eng.run_host_top3(0, "mixed", w.t, w.y, None, offs, w.fmin, w.df, n_freq,
                           normalize=True, want_pgram=True)
    gidx, gpw = pyoracle.top3(t3.pgram.reshape(-1))
    np.testing.assert_array_equal(t3.best_idx[0], gidx)
    np.testing.assert_array_equal(t3.best_power[0], gpw)
