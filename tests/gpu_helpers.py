"""Shared checks of the GPU parity tests (tolerances are stated here once).

PLAIN_RTOL   per-frequency relative error of the plain FP64 form against the FP64
             oracle / the reference's CPU build (bar: 1e-9). Near-zero powers are the
             cancellation of sums of O(N) terms, so two FP64 implementations that
             round differently (CUDA sincos vs glibc, fused vs unfused adds) differ
             there by ~1e-16 * N relative to the object's peak, not to the tiny power.
             Powers below PLAIN_FLOOR * peak are therefore compared against
             PLAIN_FLOOR * peak: an absolute bar of 1e-12 of the peak.
MIXED_ATOL   absolute error of the mixed form on normalized power (bar: 1e-4).
Best periods must be identical; for the mixed form a different index is accepted
only when the oracle's powers at the two indices differ by less than the
tolerance (the top two peaks are tied within it).
"""
import numpy as np

PLAIN_RTOL = 1e-9
PLAIN_FLOOR = 1e-3
MIXED_ATOL = 1e-4


def plain_rel_err(gpu, ref):
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    peak = np.max(np.abs(ref), axis=-1, keepdims=True)
    denom = np.maximum(np.abs(ref), PLAIN_FLOOR * peak)
    return float(np.max(np.abs(gpu - ref) / denom))


def mixed_abs_err(gpu, ref):
    return float(np.max(np.abs(np.asarray(gpu, np.float64) - np.asarray(ref, np.float64))))


def check_best(gpu_idx, ref_pgram, ref_kidx=None, tol=0.0):
    """gpu_idx[o] vs argmax of ref_pgram[o] (columns are grid indices ref_kidx)."""
    ref_pgram = np.atleast_2d(ref_pgram)
    kk = np.arange(ref_pgram.shape[1]) if ref_kidx is None else np.asarray(ref_kidx)
    bad = []
    for o in range(ref_pgram.shape[0]):
        j_ref = int(np.argmax(ref_pgram[o]))
        k_ref = int(kk[j_ref])
        k_gpu = int(gpu_idx[o])
        if k_gpu == k_ref:
            continue
        pos = np.nonzero(kk == k_gpu)[0]
        if tol > 0 and pos.size and ref_pgram[o, j_ref] - ref_pgram[o, pos[0]] <= tol:
            continue
        bad.append((o, k_ref, k_gpu))
    return bad
