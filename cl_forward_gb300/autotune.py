"""Autotuned launch configurations, cached per GPU and workload shape.

The sweep itself is native (``velo_autotune`` in the C ABI): threads per
event, hits staged per shared-memory tile, register build and launch style,
then seeding lanes per h0 on the three fastest, timed on the caller's staged
events.  This module caches the winner in a JSON
file next to the built library, keyed by the device's SM count and the batch
shape (event count and mean hits, bucketed to powers of two), so repeated
runs of the same workload skip the sweep.
"""
from __future__ import annotations

import json
import math
import os
from typing import Optional, Tuple

from . import native

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune_cache.json")
FIELDS = ("threads_per_event", "launch_mode", "smem_hits", "narrow_windows", "register_ctas", "seed_lanes")


SPACE = 7   # bumped when velo_autotune's candidate set changes: older entries are ignored


def shape_key(sm_count: int, n_events: int, mean_hits: float, y_lanes: int) -> str:
    b = lambda v: 2 ** int(round(math.log2(max(v, 1))))
    return f"sm{sm_count}-ev{b(n_events)}-hits{b(mean_hits)}-y{y_lanes}-s{SPACE}"


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, table: dict) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def options_from(entry: dict, base: Optional[native.Options] = None) -> native.Options:
    o = base or native.default_options()
    for k in FIELDS:
        setattr(o, k, int(entry[k]))
    return o


def tuned_options(ctx: native.Context, n_events: int, mean_hits: float, base: Optional[native.Options] = None,
                  iters: int = 3, cache_path: str = CACHE, refresh: bool = False) -> Tuple[native.Options, dict]:
    """Options for the events staged in ``ctx`` (tuning them on a cache miss)."""
    base = base or native.default_options()
    key = shape_key(ctx.sm_count, n_events, mean_hits, base.y_lanes)
    table = _load(cache_path)
    if not refresh and key in table:
        return options_from(table[key], base), dict(table[key], key=key, cached=True)
    best, ms = ctx.autotune(base, iters)
    entry = {k: int(getattr(best, k)) for k in FIELDS}
    entry["ms"] = ms
    table[key] = entry
    _store(cache_path, table)
    return options_from(entry, base), dict(entry, key=key, cached=False)
