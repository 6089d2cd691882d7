"""Autotuner: bucketing and the cache (CPU), tuning on the GPU."""
import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import autotune
from gpu_lomb_scargle_gb300 import engine as E
from gpu_lomb_scargle_gb300 import synth


def test_bucket_is_stable_and_coarse():
    a = autotune.bucket(np.array([0, 100, 250, 400]), 1_000_000)
    b = autotune.bucket(np.array([0, 110, 240, 400]), 900_000)
    assert a == b  # nearby batches share a bucket
    assert autotune.bucket(np.array([0, 5000]), 10_000_000) != a


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("LSGB_TUNING_CACHE", str(tmp_path / "t.json"))
    assert autotune.lookup(0, "n128:f1048576:o1024") is None
    autotune._save({autotune._key(0, "n128:f1048576:o1024"): {"shape": [12, 256, 2, 1, 0]}})
    assert autotune.lookup(0, "n128:f1048576:o1024") == (12, 256, 2, 1, 0)


@pytest.mark.gpu
def test_tune_and_apply(native_libs, cuda_ok, tmp_path, monkeypatch):
    monkeypatch.setenv("LSGB_TUNING_CACHE", str(tmp_path / "t.json"))
    eng = E.Engine(0)
    w = synth.lognormal_batch(seed=3, n_obj=64, n_freq=50_000)
    ref = eng.run_host(0, "mixed", w.t, w.y, None, w.offsets, w.fmin, w.df, w.n_freq)
    shape = autotune.apply(eng, 0, w.offsets, w.n_freq)
    assert shape is not None and eng.get_tuning(0) == tuple(shape)
    assert autotune.lookup(0, autotune.bucket(w.offsets, w.n_freq)) == tuple(shape)
    r = eng.run_host(0, "mixed", w.t, w.y, None, w.offsets, w.fmin, w.df, w.n_freq)
    # another shape may round differently; best periods agree within the tolerance
    assert np.max(np.abs(r.best_power - ref.best_power)) < 1e-4
