"""lsgb_periodogram_noalloc: the periodogram for callers that must not allocate.

Some callers of this library cannot let it call cudaMalloc while they run:
* a plugin inside a host framework whose allocator owns the whole device budget;
* a latency-critical loop that cannot take the synchronization an allocation may bring;
* a service that reserves its whole footprint at start-up.
For them the library has one entry point that keeps all of its scratch (observation
records, per-object tables, per-tile maxima, the work-queue counter) in a fixed-size
array compiled into liblsgb.so. These tests call it through the C ABI and check it
against the regular entry point, lsgb_periodogram_device, with the tolerance the other
mixed-form tests use. They check two calls in a row, because every call reuses the
same array and must not see what the previous call left in it.

This file is named to be collected last, so that a run stopping at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import _native
from gpu_lomb_scargle_gb300 import engine as E
from gpu_lomb_scargle_gb300 import synth
from tests.gpu_helpers import MIXED_ATOL, mixed_abs_err


def _noalloc(lib, variant, t, y, dy, offsets, fmin, df, n_freq, normalize, pgram, best_idx,
             best_power, stream, dtype=E.F64):
    ptr = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None
    offs = np.ascontiguousarray(offsets, dtype=np.uint64)
    return lib.lsgb_periodogram_noalloc(
        int(variant), dtype, ptr(t), ptr(y), ptr(dy),
        offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), offs.size - 1, float(fmin),
        float(df), int(n_freq), int(normalize), ptr(pgram), ptr(best_idx), ptr(best_power),
        ctypes.c_void_p(stream.cuda_stream))


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1])
def test_noalloc_matches_regular_entry_point_twice(native_libs, cuda_ok, variant):
    import torch

    lib = _native.lsgb()
    eng = E.Engine(0)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream()
    # two different batches in a row: the second is smaller, so scratch written by the
    # first is still there beyond the second's extent
    batches = [synth.lognormal_batch(seed=900 + variant, n_obj=300, n_freq=40_000,
                                     error=bool(variant)),
               synth.lognormal_batch(seed=950 + variant, n_obj=57, n_freq=12_345,
                                     error=bool(variant))]
    for w in batches:
        t = torch.from_numpy(w.t).to(dev)
        y = torch.from_numpy(w.y).to(dev)
        dy = torch.from_numpy(w.dy).to(dev) if variant else None
        outs = []
        for path in ("regular", "noalloc"):
            pg = torch.full((w.n_obj, w.n_freq), -1.0, dtype=torch.float64, device=dev)
            bi = torch.full((w.n_obj,), -1, dtype=torch.int32, device=dev)
            bp = torch.full((w.n_obj,), -1.0, dtype=torch.float64, device=dev)
            if path == "regular":
                eng.run_device(variant, "mixed", t, y, dy, w.offsets, w.fmin, w.df, w.n_freq,
                               variant == 0, pg, bi, bp, stream)
            else:
                rc = _noalloc(lib, variant, t, y, dy, w.offsets, w.fmin, w.df, w.n_freq,
                              variant == 0, pg, bi, bp, stream)
                assert rc == 0, lib.lsgb_last_error().decode()
            torch.cuda.synchronize()
            outs.append((pg.cpu().numpy(), bi.cpu().numpy(), bp.cpu().numpy()))
        (pg_r, bi_r, bp_r), (pg_n, bi_n, bp_n) = outs
        assert mixed_abs_err(pg_n, pg_r) < MIXED_ATOL
        assert mixed_abs_err(bp_n, bp_r) < MIXED_ATOL
        # best frequencies agree, or their powers are tied within the tolerance
        rows = np.arange(w.n_obj)
        diff = bi_n != bi_r
        assert np.all(np.abs(pg_r[rows, bi_r] - pg_r[rows, bi_n])[diff] <= MIXED_ATOL)
        assert np.array_equal(bi_n, np.argmax(pg_n, axis=1))
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [E.F32, E.F64])
def test_noalloc_float_inputs_and_long_objects(native_libs, cuda_ok, dtype):
    """Float and double inputs, and objects longer than one shared-memory chunk of
    observations (1,024), up to near the 131,072-observation limit: such objects are summed
    in two levels, as the regular entry point sums them. Two calls in a row again."""
    import torch

    lib = _native.lsgb()
    eng = E.Engine(0)
    dev = torch.device("cuda:0")
    tdt = torch.float32 if dtype == E.F32 else torch.float64
    stream = torch.cuda.current_stream()
    long_w = synth.long_object(seed=4100, n_obs=120_000, n_freq=3_000)
    short = synth.lognormal_batch(seed=4200, n_obj=3, n_freq=3_000)
    # objects of 120,000, then 5,000 (a slice of the long one) and three short ones
    t = np.concatenate([long_w.t, long_w.t[:5000], short.t])
    y = np.concatenate([long_w.y, long_w.y[:5000], short.y])
    offs = np.concatenate([[0, 120_000, 125_000], 125_000 + short.offsets[1:]]).astype(np.uint64)
    fmin, df, nf = long_w.fmin, long_w.df, long_w.n_freq
    assert offs[-1] <= 131072
    for call in range(2):
        tt = torch.from_numpy(t).to(dev, tdt)
        yy = torch.from_numpy(y).to(dev, tdt)
        outs = []
        for path in ("regular", "noalloc"):
            pg = torch.full((offs.size - 1, nf), -1.0, dtype=tdt, device=dev)
            bi = torch.full((offs.size - 1,), -1, dtype=torch.int32, device=dev)
            bp = torch.full((offs.size - 1,), -1.0, dtype=tdt, device=dev)
            if path == "regular":
                eng.run_device(0, "mixed", tt, yy, None, offs, fmin, df, nf, True, pg, bi, bp,
                               stream)
            else:
                rc = _noalloc(lib, 0, tt, yy, None, offs, fmin, df, nf, True, pg, bi, bp, stream,
                              dtype)
                assert rc == 0, lib.lsgb_last_error().decode()
            torch.cuda.synchronize()
            outs.append((pg.double().cpu().numpy(), bi.cpu().numpy(), bp.double().cpu().numpy()))
        (pg_r, bi_r, bp_r), (pg_n, bi_n, bp_n) = outs
        assert mixed_abs_err(pg_n, pg_r) < MIXED_ATOL, call
        assert mixed_abs_err(bp_n, bp_r) < MIXED_ATOL
        rows = np.arange(offs.size - 1)
        diff = bi_n != bi_r
        assert np.all(np.abs(pg_r[rows, bi_r] - pg_r[rows, bi_n])[diff] <= MIXED_ATOL)
        y = y[::-1].copy()  # the second call sees different data in the same scratch
    eng.close()


def test_noalloc_rejects_sizes_beyond_its_limit(native_libs):
    """Sizes above the compiled limits are refused before any device work (no GPU needed)."""
    lib = _native.lsgb()
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the size check comes first

    def call(offsets, n_freq):
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        return lib.lsgb_periodogram_noalloc(
            0, E.F64, fake, fake, None, offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            offs.size - 1, 1.0, 1e-4, n_freq, 1, None, fake, fake, None)

    assert call([0, 131073], 10) == -1  # too many observations
    assert "131072 observations" in lib.lsgb_last_error().decode()
    assert call(np.arange(2050), 10) == -1  # too many objects
    assert "2048 objects" in lib.lsgb_last_error().decode()
    assert call(np.arange(0, 2001 * 10, 10), 3072 * 200) == -1  # too many tile units
    assert "262144" in lib.lsgb_last_error().decode()
