"""The continuous-batching request loop: every object's result is the same alone and in
the mix, within the mixed form's tolerance, and agrees with the oracle.

An object computed alone is a batch of few (object, frequency tile) pairs, which the tensor
form cuts into K slices when the object has 512 or more observations; in a batch with more
pairs than SMs it is not cut. The two sum in different orders, so their powers may differ in
the last bits of FP32: the comparison is within MIXED_ATOL, and the best index is the same
or a near-tie within it."""
import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import engine as E
from gpu_lomb_scargle_gb300 import serve, synth
from oracle import pyoracle
from tests.gpu_helpers import MIXED_ATOL


def same_as_alone(res, i, alone, eng, variant, t, y, dy, st):
    """Object i's result from the server against the same object computed alone."""
    assert abs(res["best_power"][i] - alone.best_power[0]) <= MIXED_ATOL, i
    if res["best_idx"][i] != alone.best_idx[0]:
        # a near-tie: the alone periodogram's powers at the two indices are within the bar
        df = (st.fmax - st.fmin) / st.n_freq
        pg = eng.run_host(variant, "mixed", t, y, dy if variant else None,
                          np.array([0, t.size], np.uint64), st.fmin, df, st.n_freq,
                          normalize=True, want_pgram=True).pgram.reshape(-1)
        assert abs(pg[res["best_idx"][i]] - pg[alone.best_idx[0]]) <= MIXED_ATOL, i


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1])
def test_results_alone_equal_results_in_the_mix(native_libs, cuda_ok, variant):
    st = synth.stream(seed=77 + variant, n_obj=500, rate_hz=5000.0, n_freq=20_000)
    rng = np.random.default_rng(5)
    objects = []
    for i in range(500):
        t, y = synth.stream_object(st, i)
        dy = rng.uniform(0.01, 0.1, t.size) if variant else np.ones_like(t)
        objects.append((t, y, dy))
    report, res = serve.replay(st, variant=variant, slots=3, max_batch=64, objects=objects)
    assert report["completed"] == 500
    assert report["batches"] > 3  # arrivals were spread over several overlapping batches
    eng = E.Engine(0)
    df = (st.fmax - st.fmin) / st.n_freq
    for i, (t, y, dy) in enumerate(objects):
        alone = eng.run_host(variant, "mixed", t, y, dy if variant else None,
                             np.array([0, t.size], np.uint64), st.fmin, df, st.n_freq,
                             normalize=True)
        assert res["ids"][i] == i
        same_as_alone(res, i, alone, eng, variant, t, y, dy, st)
    # and a sample against the oracle (grid indices around each best and a coarse sweep)
    for i in range(0, 500, 50):
        t, y, dy = objects[i]
        if variant:
            _, y = pyoracle.batch_pgram(1, t, y, dy, [0, t.size], st.fmin, df, n_freq=1)
        kk = np.unique(np.concatenate([np.arange(0, st.n_freq, 97),
                                       np.clip(res["best_idx"][i] + np.arange(-5, 6), 0,
                                               st.n_freq - 1)]))
        ref, _ = pyoracle.batch_pgram(variant, t, y, dy, [0, t.size], st.fmin, df, kidx=kk)
        k = int(res["best_idx"][i])
        assert abs(ref[0][np.searchsorted(kk, k)] - res["best_power"][i]) < MIXED_ATOL
        assert ref[0].max() - ref[0][np.searchsorted(kk, k)] <= MIXED_ATOL


def test_server_without_gpu_fails_loudly(native_libs):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(E.LsgbError) as ei:
        serve.Server(1000, 1.0, 1e-3)
    assert ei.value.status == -4


@pytest.mark.gpu
def test_admission_under_a_binding_hbm_budget(native_libs, cuda_ok):
    """Arrivals faster than the GPU serves them, and an HBM budget of about two batches:
    admissions stop at the budget and objects wait, several batches are in flight at once,
    and every result is still the same as the object computed alone."""
    st = synth.stream(seed=91, n_obj=1500, rate_hz=60_000.0, n_freq=100_000)
    objects = []
    for i in range(1500):
        t, y = synth.stream_object(st, i)
        objects.append((t, y, np.ones_like(t)))
    # device bytes in flight (lsgb_server.cpp batch_footprint): about 5.4 KB for an average
    # object at 1e5 frequencies, so a 64 KB budget holds a dozen of them at a time
    budget = 64 * 1024
    report, res = serve.replay(st, slots=3, max_batch=64, hbm_budget_bytes=budget,
                               objects=objects)
    print({k: report[k] for k in ("batches", "largest_batch", "peak_slots_in_flight",
                                  "peak_waiting", "budget_deferrals", "peak_inflight_bytes",
                                  "latency_p50_ms", "latency_p99_ms")})
    assert report["completed"] == 1500
    assert report["budget_deferrals"] > 0
    assert report["peak_waiting"] > 1
    assert report["peak_slots_in_flight"] >= 2
    assert report["peak_inflight_bytes"] <= budget or report["largest_batch"] == 1
    eng = E.Engine(0)
    df = (st.fmax - st.fmin) / st.n_freq
    for i in range(0, 1500, 7):
        t, y, _ = objects[i]
        alone = eng.run_host(0, "mixed", t, y, None, np.array([0, t.size], np.uint64), st.fmin,
                             df, st.n_freq, normalize=True)
        same_as_alone(res, i, alone, eng, 0, t, y, None, st)
    eng.close()
