"""The three best frequencies per object, found in the periodogram kernels
(lsgb_periodogram_top3_host / _device) against the reference's three scans over the oracle's
periodogram (source/main.cu:1165-1219, restated in oracle/ls_oracle.c lso_top3).

Plain FP64 form: identical indices, powers within 1e-9 relative. Mixed forms (tensor-core
default and the CUDA-core shapes): powers within 1e-4 absolute (normalized), and an index may
differ from the oracle's only where the oracle's powers at the two indices are within 1e-4.
"""
import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import engine as E
from gpu_lomb_scargle_gb300 import synth
from oracle import pyoracle
from tests.gpu_helpers import MIXED_ATOL, PLAIN_RTOL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(native_libs, cuda_ok):
    e = E.Engine(0)
    yield e
    e.close()


def oracle_top3(ref):
    idx = np.zeros((ref.shape[0], 3), np.int64)
    pw = np.zeros((ref.shape[0], 3))
    for o in range(ref.shape[0]):
        i, p = pyoracle.top3(ref[o])
        idx[o], pw[o] = i, p
    return idx, pw


def check_top3(idx, pw, ref, precision):
    ridx, rpw = oracle_top3(ref)
    if precision == "plain":
        np.testing.assert_array_equal(idx, ridx)
        np.testing.assert_allclose(pw, rpw, rtol=PLAIN_RTOL, atol=0)
        return
    np.testing.assert_allclose(pw, rpw, atol=MIXED_ATOL, rtol=0)
    for o, r in zip(*np.nonzero(idx != ridx)):
        # a near-tie: the oracle's power where the GPU chose is within the bar of its choice
        assert abs(ref[o, idx[o, r]] - rpw[o, r]) <= MIXED_ATOL, (o, r, idx[o], ridx[o])


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_top3_host_matches_three_scans(eng, variant, precision):
    w = synth.lognormal_batch(seed=77 + variant, n_obj=40, n_freq=9000, error=bool(variant))
    y = w.y
    if variant == 1:
        _, y = pyoracle.batch_pgram(1, w.t, w.y, w.dy, w.offsets, w.fmin, w.df, n_freq=1)
    ref, _ = pyoracle.batch_pgram(variant, w.t, y, w.dy, w.offsets, w.fmin, w.df, n_freq=w.n_freq)
    r = eng.run_host_top3(variant, precision, w.t, y, w.dy if variant else None, w.offsets, w.fmin,
                          w.df, w.n_freq, normalize=(variant == 0), want_pgram=True)
    assert r.best_idx.shape == (w.n_obj, 3)
    check_top3(r.best_idx.astype(np.int64), r.best_power, ref, precision)
    # the first of the three is the argmax entry point's answer, bit for bit
    r1 = eng.run_host(variant, precision, w.t, y, w.dy if variant else None, w.offsets, w.fmin,
                      w.df, w.n_freq, normalize=(variant == 0))
    np.testing.assert_array_equal(r.best_idx[:, 0], r1.best_idx)
    np.testing.assert_array_equal(r.best_power[:, 0], r1.best_power)


@pytest.mark.parametrize("shape", [(12, 256, 2, 2, 0), (12, 128, 4, 1, 0)])
def test_top3_cuda_core_shapes(native_libs, cuda_ok, shape):
    e = E.Engine(0)
    try:
        e.set_tuning(0, *shape)
        w = synth.lognormal_batch(seed=5, n_obj=25, n_freq=7000)
        ref, _ = pyoracle.batch_pgram(0, w.t, w.y, None, w.offsets, w.fmin, w.df, n_freq=w.n_freq)
        r = e.run_host_top3(0, "mixed", w.t, w.y, None, w.offsets, w.fmin, w.df, w.n_freq)
        check_top3(r.best_idx.astype(np.int64), r.best_power, ref, "mixed")
    finally:
        e.close()


def test_top3_padding_with_few_positive_powers(eng):
    """Fewer than three frequencies: the missing entries are (index 0, power 0), as the
    reference's scans leave them."""
    w = synth.lognormal_batch(seed=9, n_obj=3, n_freq=2)
    for precision in ("plain", "mixed"):
        r = eng.run_host_top3(0, precision, w.t, w.y, None, w.offsets, w.fmin, w.df, 2)
        ref, _ = pyoracle.batch_pgram(0, w.t, w.y, None, w.offsets, w.fmin, w.df, n_freq=2)
        ridx, rpw = oracle_top3(ref)
        np.testing.assert_array_equal(r.best_idx[:, 2], 0)
        np.testing.assert_array_equal(r.best_power[:, 2], 0)
        np.testing.assert_array_equal(r.best_idx[:, :2], ridx[:, :2])


def test_top3_device_entry_point(eng):
    import torch
    w = synth.lognormal_batch(seed=13, n_obj=30, n_freq=20000)
    dev = torch.device("cuda:0")
    t = torch.tensor(w.t, device=dev)
    y = torch.tensor(w.y, device=dev)
    idx = torch.zeros((w.n_obj, 3), dtype=torch.int32, device=dev)
    pw = torch.zeros((w.n_obj, 3), dtype=torch.float64, device=dev)
    eng.run_device_top3(0, "mixed", t, y, None, w.offsets, w.fmin, w.df, w.n_freq, top_idx=idx,
                        top_power=pw)
    torch.cuda.synchronize()
    ref, _ = pyoracle.batch_pgram(0, w.t, w.y, None, w.offsets, w.fmin, w.df, n_freq=w.n_freq)
    check_top3(idx.cpu().numpy().astype(np.int64), pw.cpu().numpy(), ref, "mixed")
