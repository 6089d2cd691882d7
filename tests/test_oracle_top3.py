"""The oracle's three-scan top three (oracle/ls_oracle.c lso_top3, source/main.cu:1165-1219)
equals the rule the kernels implement: the three largest (power, lowest index) pairs among
the positive powers, padded with (index 0, power 0). Exhaustive over small random cases with
ties, zeros and negative powers."""
import numpy as np

from oracle import pyoracle


def key_rule(p):
    cand = sorted((-v, i) for i, v in enumerate(p) if v > 0)[:3]
    idx = [c[1] for c in cand] + [0] * (3 - len(cand))
    pw = [-c[0] for c in cand] + [0.0] * (3 - len(cand))
    return idx, pw


def test_three_scans_equal_key_rule():
    rng = np.random.default_rng(1)
    for trial in range(3000):
        n = int(rng.integers(1, 12))
        if trial % 2:
            p = rng.choice([-1.0, 0.0, 0.5, 1.0, 2.0, 3.0], size=n)
        else:
            p = rng.normal(size=n)
        idx, pw = pyoracle.top3(p)
        e_idx, e_pw = key_rule(p)
        assert list(idx) == e_idx and np.allclose(pw, e_pw), (p, idx, pw)
