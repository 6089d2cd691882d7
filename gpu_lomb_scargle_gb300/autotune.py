"""Autotuner of the mixed kernel's shape, cached per (observation bucket, frequency bucket).

The mixed kernel is compiled in several shapes (``engine.mixed_shapes()``): frequencies
per thread F, threads per CTA, the register budget (minimum CTAs per SM), the inner loop
(scalar, packed f32x2 rotation, packed strided second-order) and the observation unroll. The fastest shape depends on the batch:
  * small objects amortize the per-(object, tile) staging and epilogue over few pairs;
  * few objects with few frequencies leave SMs idle unless tiles are small.
The re-anchoring interval R is not tuned. In this design R equals F, because each
thread's frequency run starts from an exact anchor; a longer R only adds recurrence
steps and error (lsgb_set_reanchor measures that).

``tune`` times every compiled shape of a variant on a synthetic batch with the bucket's
size profile and stores the winner in a JSON cache keyed by GPU name, variant and
bucket. ``apply`` looks a batch's bucket up (tuning it first if asked) and sets the
engine's shape. Cache file: $LSGB_TUNING_CACHE, else ~/.cache/lsgb/tuning.json.
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

import numpy as np

from . import engine as E
from . import synth


def cache_path() -> Path:
    p = os.environ.get("LSGB_TUNING_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "lsgb" / "tuning.json"


def bucket(offsets, n_freq: int) -> str:
    """Bucket of a batch: the pair-weighted mean observation count and the frequency
    count, each rounded to a power of two, plus the object count rounded likewise."""
    n = np.diff(np.asarray(offsets, dtype=np.int64)).astype(np.float64)
    n_w = float(np.sum(n * n) / max(np.sum(n), 1.0))
    nb = 2 ** int(round(math.log2(max(n_w, 8.0))))
    fb = 2 ** int(math.ceil(math.log2(max(int(n_freq), 1024))))
    ob = 2 ** int(math.ceil(math.log2(max(n.size, 1))))
    return f"n{nb}:f{fb}:o{min(ob, 1024)}"


def _gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def _load() -> dict:
    p = cache_path()
    if p.exists():
        try:
            return json.loads(p.read_text())
        except (OSError, ValueError):
            return {}
    return {}


def _save(d: dict):
    p = cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
    tmp.replace(p)


def _key(variant: int, b: str) -> str:
    return f"{_gpu_name()}|v{variant}|{b}"


def _synthetic(b: str, variant: int):
    nb, fb, ob = (int(x[1:]) for x in b.split(":"))
    n_freq = min(fb, 1 << 18)  # timing sample; the shape ranking does not need the full grid
    n_obj = max(1, min(ob, 512))
    rng = np.random.default_rng(nb * 7 + fb)
    sizes = np.clip(rng.lognormal(math.log(nb), 0.3, n_obj).round(), 4, None).astype(np.int64)
    ts, ys, dys = [], [], []
    for n in sizes:
        t = np.sort(rng.uniform(0, 1800, int(n)))
        ts.append(t)
        ys.append(np.sin(2 * np.pi * t / 0.7) + rng.normal(0, 0.3, t.size))
        dys.append(rng.uniform(0.01, 0.1, t.size))
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    return (np.concatenate(ts), np.concatenate(ys), np.concatenate(dys), offs, 1.005,
            (150.796 - 1.005) / n_freq, n_freq)


def tune(eng: E.Engine, variant: int, b: str, repeats: int = 3) -> tuple:
    """Time every compiled shape of `variant` on bucket `b`; cache and return the best."""
    import torch

    t, y, dy, offs, fmin, df, n_freq = _synthetic(b, variant)
    dev = torch.device("cuda", eng.device)
    tt = torch.from_numpy(t).to(dev)
    yy = torch.from_numpy(y).to(dev)
    dd = torch.from_numpy(dy).to(dev) if variant else None
    n_obj = offs.size - 1
    bi = torch.empty(n_obj, dtype=torch.int32, device=dev)
    bp = torch.empty(n_obj, dtype=torch.float64, device=dev)
    saved = eng.get_tuning(variant)
    results = {}
    try:
        for sh in E.mixed_shapes():
            if sh[0] != variant:
                continue
            eng.set_tuning(variant, *sh[1:])
            ms = []
            for _ in range(repeats + 1):
                eng.run_device(variant, "mixed", tt, yy, dd, offs, fmin, df, n_freq, True, None, bi,
                               bp)
                ms.append(eng.last_kernel_ms())
            results[sh[1:]] = float(np.median(ms[1:]))
    finally:
        eng.set_tuning(variant, *saved)
    best = min(results, key=results.get)
    cache = _load()
    cache[_key(variant, b)] = {"shape": list(best), "ms": results[best],
                               "candidates": {",".join(map(str, k)): v for k, v in results.items()}}
    _save(cache)
    return best


def lookup(variant: int, b: str):
    entry = _load().get(_key(variant, b))
    return tuple(entry["shape"]) if entry else None


def apply(eng: E.Engine, variant: int, offsets, n_freq: int, tune_if_missing: bool = True):
    """Set the engine's shape for this batch's bucket; returns the shape used."""
    b = bucket(offsets, n_freq)
    shape = lookup(variant, b)
    if shape is None and tune_if_missing:
        shape = tune(eng, variant, b)
    if shape is not None:
        eng.set_tuning(variant, *shape)
    return shape
