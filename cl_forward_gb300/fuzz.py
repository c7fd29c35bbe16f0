"""Small adversarial events for parity edge cases.

Hits sit on a coarse x/y grid so that extrapolation fits tie exactly, module
occupancies are ragged (empty modules included), and a few hits share x
within a module (sort ties).  Layout and geometry follow
:mod:`cl_forward_gb300.generator`, but there is no physics: the point is to
exercise the reference's tie-breaking (lowest Y-lane, then h1 order, then h2
order: Kernel.cl:302-305,517-545), the lane that stops at the first h1
without an h2 window (Kernel.cl:437,457), skipped modules and weak tracks
(Kernel.cl:349-363,771-815).
"""
from __future__ import annotations

import numpy as np

from .events import Event, pack_event
from .generator import MODULE_Z, N_MODULES


def fuzz_event(seed: int, n_modules: int = N_MODULES, max_per_module: int = 12,
               grid: float = 0.05, lines: int = 6, jitter_z: bool = False,
               x_span: float = 25.0) -> bytes:
    rng = np.random.Generator(np.random.PCG64(seed))
    S = int(n_modules)
    zmod = MODULE_Z[:S] if S <= N_MODULES else np.arange(S, dtype=np.float64) * 20.0 - 300.0
    mods, xs, ys, zs = [], [], [], []
    # a few straight lines so that seeds and forwarding happen at all
    for _ in range(lines):
        x0, y0 = rng.uniform(-20, 20, 2)
        tx, ty = rng.uniform(-0.02, 0.02, 2)
        side = rng.integers(0, 2)
        for m in range(side, S, 2):
            if rng.random() < 0.85:
                mods.append(m)
                xs.append(np.round((x0 + tx * zmod[m]) / grid) * grid)
                ys.append(np.round((y0 + ty * zmod[m]) / grid) * grid)
                zs.append(zmod[m])
    # random grid hits, ragged occupancy
    for m in range(S):
        k = int(rng.integers(0, max_per_module + 1)) if rng.random() > 0.1 else 0
        for _ in range(k):
            mods.append(m)
            xs.append(np.round(rng.uniform(-x_span, x_span) / grid) * grid)
            ys.append(np.round(rng.uniform(-25, 25) / grid) * grid)
            zs.append(zmod[m] + (np.round(rng.uniform(-1, 1), 1) if jitter_z else 0.0))
    mods = np.array(mods, np.int64)
    order = np.argsort(mods, kind="stable")
    mods = mods[order]
    counts = np.bincount(mods, minlength=S).astype(np.int32)
    starts = np.zeros(S, np.int32)
    if S:
        starts[1:] = np.cumsum(counts)[:-1]
    perm = rng.permutation(len(mods))   # shuffle within modules: unsorted like the input files
    out_order = np.lexsort((perm, mods))
    H = len(mods)
    ev = Event(
        sensor_z=np.trunc(zmod).astype(np.int32),
        hit_start=starts,
        hit_num=counts,
        hit_id=((np.arange(H, dtype=np.uint64) + 1) << np.uint64(8) | mods.astype(np.uint64)).astype(np.uint32),
        x=np.array(xs, np.float32)[order][out_order] if H else np.zeros(0, np.float32),
        y=np.array(ys, np.float32)[order][out_order] if H else np.zeros(0, np.float32),
        z=np.array(zs, np.float32)[order][out_order] if H else np.zeros(0, np.float32),
    )
    return pack_event(ev)


def empty_event(n_modules: int = N_MODULES) -> bytes:
    S = n_modules
    ev = Event(np.trunc(MODULE_Z[:S]).astype(np.int32), np.zeros(S, np.int32), np.zeros(S, np.int32),
               np.zeros(0, np.uint32), np.zeros(0, np.float32), np.zeros(0, np.float32),
               np.zeros(0, np.float32))
    return pack_event(ev)


def crowded_event(seed: int, n_hits: int, module: int = 20, base_seed: int = 9500) -> bytes:
    """A fuzz event whose module `module` holds `n_hits` uniformly spread hits
    (on a 0.05 mm grid, x and y in [-40, 40] mm) in place of its own: the
    occupancy limit of one module (VELO_MAX_MODULE_HITS) and one past it."""
    from .events import unpack_event
    base = unpack_event(fuzz_event(base_seed, max_per_module=8, grid=0.5, lines=8))
    rng = np.random.Generator(np.random.PCG64(seed))
    S = base.n_sensors
    mod_of = base.module_of_hit()
    keep = mod_of != module
    new_x = np.round(rng.uniform(-40, 40, n_hits) / 0.05) * 0.05
    new_y = np.round(rng.uniform(-40, 40, n_hits) / 0.05) * 0.05
    mods = np.concatenate([mod_of[keep], np.full(n_hits, module)])
    xs = np.concatenate([base.x[keep], new_x.astype(np.float32)])
    ys = np.concatenate([base.y[keep], new_y.astype(np.float32)])
    zs = np.concatenate([base.z[keep], np.full(n_hits, MODULE_Z[module], np.float32)])
    order = np.argsort(mods, kind="stable")
    mods = mods[order]
    counts = np.bincount(mods, minlength=S).astype(np.int32)
    starts = np.zeros(S, np.int32)
    starts[1:] = np.cumsum(counts)[:-1]
    H = len(mods)
    ev = Event(sensor_z=base.sensor_z.copy(), hit_start=starts, hit_num=counts,
               hit_id=((np.arange(H, dtype=np.uint64) + 1) << np.uint64(8) | mods.astype(np.uint64)).astype(np.uint32),
               x=xs[order].astype(np.float32), y=ys[order].astype(np.float32), z=zs[order].astype(np.float32))
    return pack_event(ev)
