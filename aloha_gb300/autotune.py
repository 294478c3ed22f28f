"""Autotuner of the batched render with a JSON cache.

The persistent batched kernel comes in four ray-tile shapes (8x4, 8x8, 16x8
and 32x4 pixels per warp chunk), each with direct stencil loads, direct loads
with the march loop written out two steps per trip, or the next sample's
stencil rows staged in shared memory; ``aloha_batch_autotune`` times all
twelve on the batch itself with CUDA events and keeps the fastest.
This module caches that choice per (GPU, batch configuration) in a JSON file
so later processes skip the sweep.
"""
from __future__ import annotations

import json
import os
import threading

_LOCK = threading.Lock()


def cache_path() -> str:
    return os.environ.get("ALOHA_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "aloha_gb300", "autotune.json"))


def batch_key(gpu_name: str, sizes, n_bricks: int, n_ranks: int, n_tf: int) -> str:
    """Cache key: GPU, the multiset of view sizes, bricks, ranks and TF size."""
    hist = {}
    for w, h in sizes:
        hist[f"{w}x{h}"] = hist.get(f"{w}x{h}", 0) + 1
    views = ",".join(f"{k}*{hist[k]}" for k in sorted(hist))
    return f"{gpu_name}|{views}|b{n_bricks}|r{n_ranks}|tf{n_tf}"


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(batch, key: str, stream=None, reps: int = 2, path: str | None = None) -> dict:
    """Apply the cached tile shape, staging and unroll for `key`, or sweep, apply and cache them."""
    path = path or cache_path()
    with _LOCK:
        entry = _load(path).get(key)
    if entry:
        batch.set_staging(entry.get("staging", 0))
        batch.set_unroll(entry.get("unroll", 1))
        batch.set_config(entry["tile_w"], entry["tile_h"], 0)
        return dict(entry, cached=True)
    w, h, ms = batch.autotune(stream, reps=reps)
    entry = {"tile_w": w, "tile_h": h, "staging": batch.staging(), "unroll": batch.unroll(), "ms": ms}
    with _LOCK:
        data = _load(path)
        data[key] = entry
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    return dict(entry, cached=False)
