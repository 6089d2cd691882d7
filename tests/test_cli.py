"""lsgb_main, the command-line front end, in the reference's two syntaxes (CPU modes
here; the GPU modes are in tests/test_gpu_dropin.py)."""
import os
import subprocess

import numpy as np
import pytest

from gpu_lomb_scargle_gb300 import _native
from oracle import pyoracle

TWO_PI = 2.0 * np.pi


def write_data(path, ids, t, y, dy=None):
    with open(path, "w") as f:
        for i in range(t.size):
            if dy is None:
                f.write(f"{ids[i]}, {t[i]:.9f}, {y[i]:.9f}\n")
            else:
                f.write(f"{ids[i]}, {t[i]:.9f}, {y[i]:.9f}, {dy[i]:.9f}\n")


def run_cli(args, cwd):
    exe = _native.LIB_DIR / "lsgb_main"
    env = dict(os.environ, LSGB_NO_STATS="1")
    return subprocess.run([str(exe), *args], cwd=cwd, capture_output=True, text=True, env=env)


def test_paper_syntax_cpu_single_object(native_libs, golden, tmp_path):
    t, y = golden["8205_std_t"], golden["8205_std_y"]
    write_data(tmp_path / "obj.txt", np.full(t.size, 8205), t, y)
    lo, hi, nf = 3.14159, 150.79645, 4000
    p = run_cli(["obj.txt", str(lo), str(hi), str(nf), "5", "-pf", "best.txt", "-ppf", "pg.txt"],
                tmp_path)
    assert p.returncode == 0, p.stderr
    assert "[Validation] Period:" in p.stdout
    # file values are printed with 9 decimals: recompute the oracle on the same rounded input
    d = np.loadtxt(tmp_path / "obj.txt", delimiter=",")
    ref, _ = pyoracle.batch_pgram(0, d[:, 1], d[:, 2], None, [0, t.size], lo, (hi - lo) / nf,
                                  n_freq=nf)
    k = int(np.argmax(ref[0]))
    row = open(tmp_path / "best.txt").read().strip().split(",")
    assert int(row[0]) == 8205
    assert abs(float(row[1]) - TWO_PI / (lo + k * (hi - lo) / nf)) < 1e-5
    pg = np.array([float(v) for v in open(tmp_path / "pg.txt").read().split(",")[1:-1]])
    assert pg.size == nf
    np.testing.assert_allclose(pg, ref[0], rtol=1e-3, atol=1e-4)  # the file keeps 4 digits


def test_release_syntax_cpu_batch_with_error(native_libs, golden, tmp_path):
    ids, t, y, dy = (golden["batch_gen_ids"], golden["batch_gen_t"], golden["batch_gen_y"],
                     golden["batch_gen_dy"])
    write_data(tmp_path / "batch.txt", ids, t, y, dy)
    lo, hi, nf = golden["batch_gen_grid"]
    p = run_cli(["-f", "batch.txt", "-min", repr(float(lo)), "-max", repr(float(hi)), "-fq", str(int(nf)), "-m",
                 "3", "-e", "-d", "-pf", "best.txt", "--top3", "top3.txt"], tmp_path)
    assert p.returncode == 0, p.stderr
    d = np.loadtxt(tmp_path / "batch.txt", delimiter=",")
    offs = np.concatenate([[0], np.nonzero(np.diff(d[:, 0]))[0] + 1, [d.shape[0]]])
    ref, _ = pyoracle.batch_pgram(1, d[:, 1], d[:, 2], d[:, 3], offs, lo, (hi - lo) / nf,
                                  n_freq=int(nf))
    best = np.loadtxt(tmp_path / "best.txt", delimiter=",")
    assert best.shape == (12, 3)
    k = np.argmax(ref, axis=1)
    np.testing.assert_allclose(best[:, 1], TWO_PI / (lo + k * (hi - lo) / nf), rtol=1e-6)
    np.testing.assert_allclose(best[:, 2], ref.max(axis=1), rtol=1e-5)
    top3 = np.loadtxt(tmp_path / "top3.txt", delimiter=",")
    assert top3.shape == (12, 7)
    assert np.all(top3[:, 4] >= top3[:, 5]) and np.all(top3[:, 5] >= top3[:, 6])


def test_usage_errors(native_libs, tmp_path):
    assert run_cli([], tmp_path).returncode == 2
    assert run_cli(["-f", "x.txt", "-m", "9", "-min", "1", "-max", "2", "-fq", "3"],
                   tmp_path).returncode == 2
    p = run_cli(["missing.txt", "1", "2", "10", "5"], tmp_path)
    assert p.returncode == 1 and "cannot open" in p.stderr
    p = run_cli(["x.txt", "np.float64(1.0)", "2", "10", "5"], tmp_path)
    assert p.returncode == 2 and "not a number" in p.stderr
