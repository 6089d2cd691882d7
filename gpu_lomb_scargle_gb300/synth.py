"""Seeded synthetic light curves with the shapes of the reference's benchmark inputs.

The reference measures its batch path on a 999-object file with log-normal
observation counts (``data/normalized_alltargs.200724_1_log_normal_obs.dat``,
165,221 rows, README.md:63-78) that is not distributed with it, and its single-object
path on a 3,555-observation object (``data/8205_normalized.txt``). These generators
produce seeded stand-ins of the same shapes, value ranges and size distributions:

* ``single_object``      -- 3,555 sorted times in [0, 1800] d, one sinusoid + N(0, 0.1^2),
                            z-scored, 1e5 angular frequencies in [1.005, 150.796].
* ``lognormal_batch``    -- 999 objects, n ~ round(LogNormal(ln 150, 0.6)) clipped to
                            [20, 1500], each generated like the single object with its own
                            seed (base + object index); 1e6 frequencies.
* ``lognormal_batch_dmag`` -- same layout with dmag ~ U[0.01, 0.1] and
                            y = 0.5 sin + 0.3 + N(0, dmag^2) (generalized variant).
* ``long_object``        -- 200,000 times in [0, 3650] d, two sinusoids (P2 = 7.3 P1,
                            amplitudes 1.0 / 0.4) + N(0, 0.2^2); 1e7 frequencies in [0.01, 150.8].
* ``stream``             -- arrival times (Poisson, 2,000 objects/s) and sizes
                            (round(LogNormal(ln 80, 0.8)) clipped to [10, 1000]) of the
                            serving workload; objects drawn lazily by ``stream_object``.

Everything is float64 and uses ``numpy.random.default_rng``; the row layout is the
reference's: contiguous runs of equal object id, ids 0..K-1 (source/lombscarglegpu.py:270-271).
"""
from __future__ import annotations

import dataclasses

import numpy as np

TWO_PI = 2.0 * np.pi


@dataclasses.dataclass
class Workload:
    """A batch of objects in the reference's row layout plus its frequency grid.

    ``fmin``/``fmax`` are angular (rad/day), ``fmax`` exclusive; the grid is
    ``omega_k = fmin + k * (fmax - fmin) / n_freq`` (source/main.cu:1364, :1611).
    """

    name: str
    obj_id: np.ndarray  # uint32 [rows]
    t: np.ndarray  # float64 [rows]
    y: np.ndarray  # float64 [rows]
    dy: np.ndarray  # float64 [rows] (ones for the standard variant)
    fmin: float
    fmax: float
    n_freq: int
    error: bool
    seed: int

    @property
    def n_rows(self) -> int:
        return int(self.t.size)

    @property
    def offsets(self) -> np.ndarray:
        """Row offsets of the objects, length n_obj + 1 (contiguous-run segmentation)."""
        change = np.nonzero(np.diff(self.obj_id.astype(np.int64)))[0] + 1
        return np.concatenate([[0], change, [self.obj_id.size]]).astype(np.int64)

    @property
    def n_obj(self) -> int:
        return int(self.offsets.size - 1)

    @property
    def pairs(self) -> int:
        """Observation x frequency pairs, the unit of work."""
        return int(self.n_rows) * int(self.n_freq)

    @property
    def df(self) -> float:
        return (self.fmax - self.fmin) / (self.n_freq * 1.0)

    def subset_freqs(self, n_freq: int) -> "Workload":
        """The first ``n_freq`` frequencies of the same grid (same df)."""
        w = dataclasses.replace(self)
        w.fmax = self.fmin + n_freq * self.df
        w.n_freq = int(n_freq)
        w.name = f"{self.name}[:{n_freq}f]"
        return w

    def take_objects(self, n_obj: int) -> "Workload":
        off = self.offsets
        end = int(off[min(n_obj, off.size - 1)])
        return dataclasses.replace(self, obj_id=self.obj_id[:end].copy(), t=self.t[:end].copy(),
                                   y=self.y[:end].copy(), dy=self.dy[:end].copy(),
                                   name=f"{self.name}[:{n_obj}obj]")


def _one_sinusoid(rng, n, t_max, noise, zscore=True):
    t = np.sort(rng.uniform(0.0, t_max, n))
    period = np.exp(rng.uniform(np.log(0.04), np.log(6.0)))
    phase = rng.uniform(0.0, TWO_PI)
    y = np.sin(TWO_PI * t / period + phase) + rng.normal(0.0, noise, n)
    if zscore:
        y = (y - y.mean()) / y.std()
    return t, y, period


def single_object(seed: int = 1000, n_obs: int = 3555, n_freq: int = 100_000) -> Workload:
    rng = np.random.default_rng(seed)
    t, y, _ = _one_sinusoid(rng, n_obs, 1800.0, 0.1)
    return Workload("single_3555obs", np.zeros(n_obs, np.uint32), t, y, np.ones(n_obs), 1.005,
                    150.796, n_freq, False, seed)


def lognormal_sizes(rng, n_obj, mu, sigma, lo, hi):
    return np.clip(np.round(rng.lognormal(mu, sigma, n_obj)), lo, hi).astype(np.int64)


def lognormal_batch(seed: int = 2000, n_obj: int = 999, n_freq: int = 1_000_000,
                    error: bool = False) -> Workload:
    rng = np.random.default_rng(seed)
    sizes = lognormal_sizes(rng, n_obj, np.log(150.0), 0.6, 20, 1500)
    ts, ys, dys, ids = [], [], [], []
    for o, n in enumerate(sizes):
        r = np.random.default_rng(seed + 1 + o)
        if not error:
            t, y, _ = _one_sinusoid(r, int(n), 1800.0, 0.1)
            dy = np.ones(int(n))
        else:
            t = np.sort(r.uniform(0.0, 1800.0, int(n)))
            period = np.exp(r.uniform(np.log(0.04), np.log(6.0)))
            phase = r.uniform(0.0, TWO_PI)
            dy = r.uniform(0.01, 0.1, int(n))
            y = 0.5 * np.sin(TWO_PI * t / period + phase) + 0.3 + r.normal(0.0, 1.0, int(n)) * dy
        ts.append(t)
        ys.append(y)
        dys.append(dy)
        ids.append(np.full(int(n), o, np.uint32))
    name = "lognormal_%dobj_%s" % (n_obj, "dmag" if error else "std")
    return Workload(name, np.concatenate(ids), np.concatenate(ts), np.concatenate(ys),
                    np.concatenate(dys), 1.005, 150.796, n_freq, error, seed)


def lognormal_batch_dmag(seed: int = 3000, n_obj: int = 999, n_freq: int = 1_000_000) -> Workload:
    return lognormal_batch(seed, n_obj, n_freq, error=True)


def long_object(seed: int = 4000, n_obs: int = 200_000, n_freq: int = 10_000_000) -> Workload:
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0.0, 3650.0, n_obs))
    p1 = np.exp(rng.uniform(np.log(0.05), np.log(2.0)))
    p2 = 7.3 * p1
    ph1, ph2 = rng.uniform(0.0, TWO_PI, 2)
    y = (np.sin(TWO_PI * t / p1 + ph1) + 0.4 * np.sin(TWO_PI * t / p2 + ph2)
         + rng.normal(0.0, 0.2, n_obs))
    return Workload("long_200kobs", np.zeros(n_obs, np.uint32), t, y, np.ones(n_obs), 0.01, 150.8,
                    n_freq, False, seed)


@dataclasses.dataclass
class Stream:
    """Arrival process of the serving workload: arrival[i] seconds, size[i] observations."""

    arrival: np.ndarray
    size: np.ndarray
    seed: int
    fmin: float = 1.005
    fmax: float = 150.796
    n_freq: int = 200_000


def stream(seed: int = 5000, n_obj: int = 100_000, rate_hz: float = 2000.0,
           n_freq: int = 200_000) -> Stream:
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, n_obj)
    sizes = lognormal_sizes(rng, n_obj, np.log(80.0), 0.8, 10, 1000)
    return Stream(np.cumsum(gaps), sizes, seed, n_freq=n_freq)


def stream_object(s: Stream, i: int):
    """Observations (t, y) of object i of a stream, generated like the single object."""
    r = np.random.default_rng(s.seed + 1 + i)
    t, y, _ = _one_sinusoid(r, int(s.size[i]), 1800.0, 0.1)
    return t, y
