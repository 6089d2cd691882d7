"""lsgb_main, the command-line front end, in the reference's two syntaxes.

The reference's programs write the standard periodogram unnormalized unless asked
(source/params.h:40 NORMALIZEPGRAM 0; release/main.cu:376 -nrp), take the CPU thread count
with -n (release/main.cu:330), and write the three best periods with the three-scan rule of
source/main.cu:1165-1219. The CPU modes run here; the GPU modes (MODE 1 / 2) are marked gpu.
Every value is checked against the oracle on the same (text-rounded) input.
"""
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
                f.write(f"{int(ids[i])}, {float(t[i])!r}, {float(y[i])!r}\n")
            else:
                f.write(f"{int(ids[i])}, {float(t[i])!r}, {float(y[i])!r}, {float(dy[i])!r}\n")


def run_cli(args, cwd, env_extra=None):
    exe = _native.LIB_DIR / "lsgb_main"
    env = dict(os.environ, LSGB_NO_STATS="1", **(env_extra or {}))
    return subprocess.run([str(exe), *args], cwd=cwd, capture_output=True, text=True, env=env)


def load_rows(path):
    return np.atleast_2d(np.loadtxt(path, delimiter=","))


def oracle_on_file(path, variant, lo, hi, nf, normalize):
    """Oracle periodogram of the objects in a data file (its rows as the CLI read them)."""
    d = load_rows(path)
    offs = np.concatenate([[0], np.nonzero(np.diff(d[:, 0]))[0] + 1, [d.shape[0]]])
    ref, _ = pyoracle.batch_pgram(variant, d[:, 1], d[:, 2], d[:, 3] if variant else None, offs,
                                  lo, (hi - lo) / nf, n_freq=int(nf), normalize=normalize)
    return ref, d[offs[:-1], 0].astype(np.int64)


def expected_top3(ref, lo, step):
    """Periods and powers of the reference's three scans over each oracle periodogram."""
    per, pw = [], []
    for row in ref:
        idx, p = pyoracle.top3(row)
        per.append(TWO_PI / (lo + idx * step))
        pw.append(p)
    return np.array(per), np.array(pw)


def check_files(tmp_path, ref, ids, lo, hi, nf, per_rtol, pow_atol, pgram=True):
    step = (hi - lo) / nf
    best = load_rows(tmp_path / "best.txt")
    top3 = load_rows(tmp_path / "top3.txt")
    assert best.shape == (ref.shape[0], 3) and top3.shape == (ref.shape[0], 7)
    np.testing.assert_array_equal(best[:, 0].astype(np.int64), ids)
    per, pw = expected_top3(ref, lo, step)
    # six significant digits in the files (precision 6, as the reference's writers)
    np.testing.assert_allclose(best[:, 1], per[:, 0], rtol=per_rtol)
    np.testing.assert_allclose(best[:, 2], pw[:, 0], rtol=1e-5, atol=pow_atol)
    np.testing.assert_allclose(top3[:, 1:4], per, rtol=per_rtol)
    np.testing.assert_allclose(top3[:, 4:7], pw, rtol=1e-5, atol=pow_atol)
    if pgram:
        rows = open(tmp_path / "pg.txt").read().strip().split("\n")
        assert len(rows) == ref.shape[0]
        for o, line in enumerate(rows):
            vals = line.split(",")
            assert int(vals[0]) == ids[o]
            pg = np.array([float(v) for v in vals[1:-1]])
            assert pg.size == nf
            # four significant digits in the file
            np.testing.assert_allclose(pg, ref[o], rtol=1e-3,
                                       atol=max(pow_atol, 1e-4 * ref[o].max()))


def test_paper_syntax_cpu_single_object_unnormalized(native_libs, golden, tmp_path):
    t, y = golden["8205_std_t"], golden["8205_std_y"]
    write_data(tmp_path / "obj.txt", np.full(t.size, 8205), t, y)
    lo, hi, nf = 3.14159, 150.79645, 4000
    p = run_cli(["obj.txt", str(lo), str(hi), str(nf), "5", "-pf", "best.txt", "--top3", "top3.txt",
                 "-ppf", "pg.txt", "-n", "2"], tmp_path)
    assert p.returncode == 0, p.stderr
    assert "[Validation] Period:" in p.stdout
    ref, ids = oracle_on_file(tmp_path / "obj.txt", 0, lo, hi, nf, normalize=False)
    # unnormalized: the peak is O(N) (hundreds), not O(1)
    assert ref.max() > 10.0
    check_files(tmp_path, ref, ids[:1], lo, hi, nf, per_rtol=1e-5, pow_atol=1e-9)


def test_normpgram_option_normalizes(native_libs, golden, tmp_path):
    t, y = golden["8205_std_t"], golden["8205_std_y"]
    write_data(tmp_path / "obj.txt", np.full(t.size, 8205), t, y)
    lo, hi, nf = 3.14159, 150.79645, 2000
    p = run_cli(["-f", "obj.txt", "-min", str(lo), "-max", str(hi), "-fq", str(nf), "-m", "4", "-d",
                 "-nrp", "-pf", "best.txt", "--top3", "top3.txt", "-ppf", "pg.txt"], tmp_path)
    assert p.returncode == 0, p.stderr
    ref, ids = oracle_on_file(tmp_path / "obj.txt", 0, lo, hi, nf, normalize=True)
    check_files(tmp_path, ref, ids[:1], lo, hi, nf, per_rtol=1e-5, pow_atol=1e-9)


def test_release_syntax_cpu_batch_with_error(native_libs, golden, tmp_path):
    ids, t, y, dy = (golden["batch_gen_ids"], golden["batch_gen_t"], golden["batch_gen_y"],
                     golden["batch_gen_dy"])
    write_data(tmp_path / "batch.txt", ids, t, y, dy)
    lo, hi, nf = golden["batch_gen_grid"]
    lo, hi, nf = float(lo), float(hi), int(nf)
    p = run_cli(["-f", "batch.txt", "-min", repr(lo), "-max", repr(hi), "-fq", str(nf), "-m",
                 "3", "-e", "-d", "-n", "3", "-ng", "1", "-pf", "best.txt", "--top3", "top3.txt",
                 "-ppf", "pg.txt"], tmp_path)
    assert p.returncode == 0, p.stderr
    ref, oid = oracle_on_file(tmp_path / "batch.txt", 1, lo, hi, nf, normalize=False)
    check_files(tmp_path, ref, oid, lo, hi, nf, per_rtol=1e-5, pow_atol=1e-9)


def test_published_243_answer_cpu(native_libs, golden, tmp_path):
    """README.md:80-94: 243 -> period 0.096536, power 1.080289 (unnormalized, double)."""
    t, y = golden["243_t"], golden["243_y"]
    write_data(tmp_path / "243.txt", np.full(t.size, 243), t, y)
    p = run_cli(["243.txt", "3.142", "150.796", "1000000", "5"], tmp_path)
    assert p.returncode == 0, p.stderr
    assert "[Validation] Period: 0.096536, Power: 1.080289" in p.stdout, p.stdout


def test_usage_errors(native_libs, tmp_path):
    assert run_cli([], tmp_path).returncode == 2
    assert run_cli(["-f", "x.txt", "-m", "9", "-min", "1", "-max", "2", "-fq", "3"],
                   tmp_path).returncode == 2
    p = run_cli(["missing.txt", "1", "2", "10", "5"], tmp_path)
    assert p.returncode == 1 and "cannot open" in p.stderr
    p = run_cli(["x.txt", "np.float64(1.0)", "2", "10", "5"], tmp_path)
    assert p.returncode == 2 and "not a number" in p.stderr
    p = run_cli(["x.txt", "1", "2", "10", "5", "-n", "0"], tmp_path)
    assert p.returncode == 2 and "threads" in p.stderr
    p = run_cli(["x.txt", "1", "2", "10", "5", "--bogus"], tmp_path)
    assert p.returncode == 2 and "unknown option" in p.stderr


# ---- GPU modes ------------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_batch_mode_double_files_match_oracle(native_libs, cuda_ok, golden, tmp_path):
    """MODE 1 of the double build (plain FP64 form): bestperiods, top three and periodogram
    files of a 12-object batch, unnormalized, against the oracle's three scans."""
    ids, t, y = golden["batch_std_ids"], golden["batch_std_t"], golden["batch_std_y"]
    write_data(tmp_path / "batch.txt", ids, t, y)
    lo, hi, nf = golden["batch_std_grid"]
    lo, hi, nf = float(lo), float(hi), int(nf)
    p = run_cli(["batch.txt", repr(lo), repr(hi), str(nf), "1", "-pf", "best.txt", "--top3",
                 "top3.txt", "-ppf", "pg.txt"], tmp_path)
    assert p.returncode == 0, p.stderr
    assert "[Validation] Sum of all periods:" in p.stdout
    ref, oid = oracle_on_file(tmp_path / "batch.txt", 0, lo, hi, nf, normalize=False)
    check_files(tmp_path, ref, oid, lo, hi, nf, per_rtol=1e-5, pow_atol=1e-9)


@pytest.mark.gpu
def test_gpu_batch_mode_float_mixed_form(native_libs, cuda_ok, golden, tmp_path):
    """MODE 1 of the float build (mixed form), -nrp: normalized powers within 1e-4; a top-3
    index may differ from the oracle's only where the oracle's powers are tied within 1e-4."""
    ids, t, y = golden["batch_std_ids"], golden["batch_std_t"], golden["batch_std_y"]
    write_data(tmp_path / "batch.txt", ids, t, y)
    lo, hi, nf = golden["batch_std_grid"]
    lo, hi, nf = float(lo), float(hi), int(nf)
    p = run_cli(["-f", "batch.txt", "-min", repr(lo), "-max", repr(hi), "-fq", str(nf), "-m", "1",
                 "-nrp", "-pf", "best.txt", "--top3", "top3.txt", "-ppf", "pg.txt"], tmp_path)
    assert p.returncode == 0, p.stderr
    # the float build's inputs and grid, in FP64
    d = load_rows(tmp_path / "batch.txt")
    offs = np.concatenate([[0], np.nonzero(np.diff(d[:, 0]))[0] + 1, [d.shape[0]]])
    f0, step = pyoracle.float_grid(lo, hi, nf)
    ref, _ = pyoracle.batch_pgram(0, d[:, 1].astype(np.float32), d[:, 2].astype(np.float32), None,
                                  offs, f0, step, n_freq=nf, normalize=True)
    top3 = load_rows(tmp_path / "top3.txt")
    per, pw = expected_top3(ref, f0, step)
    # normalized powers within 1e-4, and the files' six significant digits
    np.testing.assert_allclose(top3[:, 4:7], pw, rtol=1e-5, atol=1e-4)
    for o in range(ref.shape[0]):
        for r in range(3):
            if abs(top3[o, 1 + r] - per[o, r]) > 1e-5 * per[o, r]:
                k_file = int(round((TWO_PI / top3[o, 1 + r] - f0) / step))
                assert abs(ref[o, k_file] - pw[o, r]) <= 1e-4, (o, r)


@pytest.mark.gpu
def test_gpu_single_mode_published_243_answer(native_libs, cuda_ok, golden, tmp_path):
    """README.md:80-94 through MODE 2 of the double build: period 0.096536, power 1.080289."""
    t, y = golden["243_t"], golden["243_y"]
    write_data(tmp_path / "243.txt", np.full(t.size, 243), t, y)
    p = run_cli(["243.txt", "3.142", "150.796", "1000000", "2", "-pf", "best.txt", "--top3",
                 "top3.txt"], tmp_path)
    assert p.returncode == 0, p.stderr
    assert "Period: 0.096536" in p.stdout and "Maximum power at found period: 1.080289" in p.stdout
    row = load_rows(tmp_path / "best.txt")[0]
    assert abs(row[1] - 0.096536) < 1e-6 and abs(row[2] - 1.080289) < 2e-6, row
    assert not (tmp_path / "pg.txt").exists()  # no -ppf: the periodogram never left the GPU


@pytest.mark.gpu
def test_gpu_single_mode_generalized_8205(native_libs, cuda_ok, golden, tmp_path):
    """README.md:120-134: 8205 with errors, 1e6 frequencies -> period 0.564736, power 0.712905."""
    t, y, dy = golden["8205_gen_t"], golden["8205_gen_y"], golden["8205_gen_dy"]
    write_data(tmp_path / "8205.txt", np.full(t.size, 8205), t, y, dy)
    p = run_cli(["8205.txt", "3.14159", "150.79645", "1000000", "2"], tmp_path)
    assert p.returncode == 0, p.stderr
    assert "[Validation] Period: 0.564736, Power: 0.712905" in p.stdout, p.stdout
