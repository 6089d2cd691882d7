"""Pin the CPU oracle (oracle/ls_oracle.c) before it is used as the checker.

Two anchors, both without a GPU:
  1. the reference's own CPU path (built from its sources, fixtures made by
     tests/golden/make_golden.py): full periodograms must agree to ~1e-12;
  2. the periods the reference publishes (README.md, python_interface_output/...).
"""
import numpy as np
import pytest

from oracle import pyoracle

TWO_PI = 2.0 * np.pi


def rel_err(a, b, floor=1e-300):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


def one(n):
    return np.array([0, n], np.int64)


@pytest.mark.parametrize("variant,tag", [(0, "8205_std"), (1, "8205_gen")])
def test_oracle_matches_reference_cpu_8205(golden, variant, tag):
    lo, hi, nf = golden["8205_grid"]
    nf = int(nf)
    t, y, dy = golden[tag + "_t"], golden[tag + "_y"], golden[tag + "_dy"]
    pg, ya = pyoracle.batch_pgram(variant, t, y, dy, one(t.size), lo, (hi - lo) / nf, n_freq=nf)
    ref = golden[tag + "_double_pgram"]
    assert rel_err(pg[0], ref) < 1e-12
    assert np.argmax(pg[0]) == np.argmax(ref)
    # generalized: y is pre-centered exactly as the reference mutates the caller's array
    np.testing.assert_allclose(ya, golden[tag + "_double_yafter"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("variant,tag", [(0, "batch_std"), (1, "batch_gen")])
def test_oracle_matches_reference_cpu_batch(golden, variant, tag):
    lo, hi, nf = golden[tag + "_grid"]
    nf = int(nf)
    ids = golden[tag + "_ids"]
    offs = np.concatenate([[0], np.nonzero(np.diff(ids))[0] + 1, [ids.size]])
    pg, ya = pyoracle.batch_pgram(variant, golden[tag + "_t"], golden[tag + "_y"],
                                  golden[tag + "_dy"], offs, lo, (hi - lo) / nf, n_freq=nf)
    ref = golden[tag + "_double_pgram"]
    assert pg.shape == ref.shape
    assert rel_err(pg, ref) < 1e-12
    assert np.array_equal(np.argmax(pg, axis=1), np.argmax(ref, axis=1))
    np.testing.assert_allclose(ya, golden[tag + "_double_yafter"], rtol=0, atol=1e-13)


def test_known_answer_243(golden):
    """README.md:82-96: 243, 29 obs, omega in [3.142, 150.796), 1e6 freqs -> P = 0.096536,
    unnormalized max power 1.080289 (the CLI build has NORMALIZEPGRAM=0)."""
    t, y = golden["243_t"], golden["243_y"]
    lo, hi, nf = 3.142, 150.796, 1_000_000
    df = (hi - lo) / nf
    k_ref, p_ref = golden["243_1e6_argmax"]
    start = int(golden["243_1e6_window_start"][0])
    win = golden["243_1e6_window"]
    kidx = np.arange(start, start + win.size)
    pg, _ = pyoracle.batch_pgram(0, t, y, None, one(t.size), lo, df, kidx=kidx)
    assert rel_err(pg[0], win) < 1e-11
    k = start + int(np.argmax(pg[0]))
    assert k == int(k_ref)
    assert round(TWO_PI / (lo + k * df), 6) == 0.096536
    # unnormalized power: divide out 2/(N var)
    norm = 2.0 / (t.size * np.var(y))
    assert round(pg[0].max() / norm, 6) == 1.080289
    # the whole 1e6 grid of a 29-observation object is cheap: the global maximum
    full, _ = pyoracle.batch_pgram(0, t, y, None, one(t.size), lo, df, n_freq=nf)
    assert int(np.argmax(full[0])) == int(k_ref)


def test_known_answer_8205_generalized_1e6(golden):
    """README.md:121-136: 8205 with dmag, omega in [3.14159, 150.79645), 1e6 freqs ->
    P = 0.564736, max power 0.712905."""
    t, y, dy = golden["8205_gen_t"], golden["8205_gen_y"], golden["8205_gen_dy"]
    lo, hi, nf = 3.14159, 150.79645, 1_000_000
    df = (hi - lo) / nf
    start = int(golden["8205_gen_1e6_window_start"][0])
    win = golden["8205_gen_1e6_window"]
    kidx = np.arange(start, start + win.size)
    pg, _ = pyoracle.batch_pgram(1, t, y, dy, one(t.size), lo, df, kidx=kidx)
    assert rel_err(pg[0], win) < 1e-11
    k = start + int(np.argmax(pg[0]))
    assert k == int(golden["8205_gen_1e6_argmax"][0])
    assert round(TWO_PI / (lo + k * df), 6) == 0.564736
    assert round(pg[0].max(), 6) == 0.712905


@pytest.mark.parametrize("variant,tag,period", [(1, "8205_gen", 0.564739), (0, "8205_std", 0.564729)])
def test_known_answer_python_example(golden, variant, tag, period):
    """python_interface_output/python_output_lomb_scargle_test_example.txt:8/16 and :24/32:
    the float Python examples (ordinary 0.1..10, 330,000 frequencies) find 0.564739
    (with dmag) and 0.564729 (without). The FP64 oracle on the same float-rounded
    inputs and float grid finds the same periods."""
    t = golden[tag + "_t"].astype(np.float32).astype(np.float64)
    y = golden[tag + "_y"].astype(np.float32).astype(np.float64)
    dy = golden[tag + "_dy"].astype(np.float32).astype(np.float64)
    nf = 330_000
    fmin, df = pyoracle.float_grid(TWO_PI * 0.1, TWO_PI * 10.0, nf)
    pg, _ = pyoracle.batch_pgram(variant, t, y, dy, one(t.size), fmin, df, n_freq=nf)
    k = int(np.argmax(pg[0]))
    df_std = (10.0 - 0.1) / nf
    assert round(1.0 / (0.1 + df_std * k), 6) == period


def test_object_ranges_contiguous_runs():
    ids = np.array([5, 5, 5, 2, 2, 9, 5, 5], np.uint32)
    lo, hi = pyoracle.object_ranges(ids)
    assert lo.tolist() == [0, 3, 5, 6]
    assert hi.tolist() == [2, 4, 5, 7]  # a non-contiguous repeat of id 5 is a new object


def test_argmax_first_maximum_rule():
    assert pyoracle.argmax([0.0, 2.0, 2.0, 1.0]) == (1, 2.0)
    assert pyoracle.argmax([-1.0, np.nan, -3.0]) == (0, 0.0)
    assert pyoracle.argmax([np.nan, 0.5, np.nan, 0.5]) == (1, 0.5)
