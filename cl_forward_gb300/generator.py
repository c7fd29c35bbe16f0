"""Seeded synthetic LHCb-VELO-like events in the search-by-triplet input layout.

The reference ships no generator (its ``mcdata/*.dat`` events carry no MC
truth), so the workloads are seeded synthetic events with this geometry:

* 26 stations, station ``s`` at ``z = -287.5 + 25 s`` mm for ``s <= 18`` and
  ``162.5 + 50 (s - 18)`` mm above; each station is a left module (x < 0) at
  ``z - 2.5`` and a right module (x > 0) at ``z + 2.5``.  Modules are indexed in
  increasing z, so even indices are left and odd indices right, and module
  ``f - 2`` is the next station on the same side (the pairing the kernel's
  h0/h1/h2 search on modules f, f-2, f-4 relies on, Kernel.cl:666-757).
* Acceptance: radius 5.1-42 mm; the two halves overlap by 1 mm across x = 0
  (left covers x < 0.5, right covers x > -0.5).
* Per event: primary vertices ~ Poisson(7.6) (or Poisson(U(a, b)) per event),
  at x, y ~ N(0, 0.05) mm and z ~ N(0, 50) mm; tracks per PV ~ Poisson(20).
  85 % of tracks have eta ~ U(1.6, 5.0), 15 % eta ~ U(-4, -2); phi uniform;
  p = 0.3 GeV + Exp(mean 5 GeV).  Straight lines with a multiple-scattering
  kick N(0, 0.5 mrad * GeV / p) on each slope after every crossed module.
  Hit efficiency 0.98, Gaussian x/y smear of 12 um, and Poisson(0.5 % of a
  module's hits) uniform noise hits per module.
* Hit IDs are ``key << 8 | module``: ``key`` is 1 + the particle index (noise
  hits get unique keys from 2**23 up), so the MC truth travels in the ID.
  Sensor z is the int32 truncation of the module z (the layout stores int32).

Hits are written per module in generation order (not x-sorted), like the
reference's input files; :func:`cl_forward_gb300.search.sort_by_x` (or
``velo_sort_by_x``) applies the reference's per-module x-sort.

Every event draws from its own ``numpy.random.Generator(PCG64(seed))`` in a
fixed order, so an event depends only on its seed and the parameters.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .events import Event, pack_event

N_STATIONS = 26
N_MODULES = 2 * N_STATIONS
R_MIN, R_MAX = 5.1, 42.0
HALF_OVERLAP = 0.5          # each half extends this far past x = 0
SIGMA_XY = 0.012            # mm
NOISE_KEY_BASE = 1 << 23


def module_z() -> np.ndarray:
    s = np.arange(N_STATIONS, dtype=np.float64)
    zs = np.where(s <= 18, -287.5 + 25.0 * s, 162.5 + 50.0 * (s - 18))
    out = np.empty(N_MODULES)
    out[0::2] = zs - 2.5      # left  (x < 0)
    out[1::2] = zs + 2.5      # right (x > 0)
    return out


MODULE_Z = module_z()
MODULE_IS_LEFT = (np.arange(N_MODULES) % 2) == 0


@dataclasses.dataclass
class GenParams:
    pv_mean: float = 7.6
    pv_mean_range: Optional[Tuple[float, float]] = None   # per-event lambda ~ U(a, b)
    tracks_per_pv: float = 20.0
    hit_eff: float = 0.98
    noise_frac: float = 0.005
    ms_mrad_gev: float = 0.5


CONFIG_SMALL = GenParams()                                   # 100 events, seeds 0..99
CONFIG_SCALE = GenParams()                                   # 10,000 events, seeds 1000..10999
CONFIG_BATCHED = GenParams(pv_mean_range=(2.0, 30.0))        # 100,000 uneven events
CONFIG_STRESS = GenParams(pv_mean=30.0, hit_eff=0.96, noise_frac=0.02)


@dataclasses.dataclass
class Truth:
    """MC truth of one event: one row per particle (key = row + 1)."""

    p: np.ndarray          # GeV
    eta: np.ndarray
    n_hits: np.ndarray     # recorded hits (after efficiency)


def _in_acceptance(x, y, left):
    r2 = x * x + y * y
    side = np.where(left, x < HALF_OVERLAP, x > -HALF_OVERLAP)
    return (r2 >= R_MIN * R_MIN) & (r2 <= R_MAX * R_MAX) & side


def _draw_tracks(rng, params: GenParams):
    """Per-event draws, in a fixed order, up to the track propagation."""
    lam = params.pv_mean
    if params.pv_mean_range is not None:
        lam = rng.uniform(params.pv_mean_range[0], params.pv_mean_range[1])
    npv = int(rng.poisson(lam))
    pv_xy = rng.normal(0.0, 0.05, (npv, 2))
    pv_z = rng.normal(0.0, 50.0, npv)
    ntrk_pv = rng.poisson(params.tracks_per_pv, npv)
    ntrk = int(ntrk_pv.sum())
    pv_of = np.repeat(np.arange(npv), ntrk_pv)
    forward = rng.random(ntrk) < 0.85
    eta_f = rng.uniform(1.6, 5.0, ntrk)
    eta_b = rng.uniform(-4.0, -2.0, ntrk)
    eta = np.where(forward, eta_f, eta_b)
    phi = rng.uniform(0.0, 2.0 * np.pi, ntrk)
    p = 0.3 + rng.exponential(5.0, ntrk)
    ms = rng.standard_normal((ntrk, N_MODULES, 2))
    eff_u = rng.random((ntrk, N_MODULES))
    smear = rng.standard_normal((ntrk, N_MODULES, 2))
    return dict(x0=pv_xy[pv_of, 0], y0=pv_xy[pv_of, 1], z0=pv_z[pv_of], forward=forward,
                eta=eta, phi=phi, p=p, ms=ms, eff_u=eff_u, smear=smear)


def _propagate(d, params: GenParams):
    """Straight lines with per-module scattering, vectorised over all tracks.

    Returns per recorded hit: (track row, module, x, y).
    """
    ntrk = d["p"].shape[0]
    theta = 2.0 * np.arctan(np.exp(-d["eta"]))
    tan_t = np.tan(theta)
    tx = tan_t * np.cos(d["phi"])
    ty = tan_t * np.sin(d["phi"])
    x = d["x0"].copy()
    y = d["y0"].copy()
    zc = d["z0"].copy()
    forward = d["forward"]
    direction = np.where(forward, 1, -1)
    start = np.where(forward, np.searchsorted(MODULE_Z, zc, side="right"),
                     np.searchsorted(MODULE_Z, zc, side="left") - 1)
    sigma = params.ms_mrad_gev * 1e-3 / d["p"]
    ms, eff_u, smear = d["ms"], d["eff_u"], d["smear"]
    idx = np.arange(ntrk)
    out_t, out_m, out_x, out_y = [], [], [], []
    for k in range(N_MODULES):
        m = start + k * direction
        alive = (m >= 0) & (m < N_MODULES)
        if not alive.any():
            break
        mm = np.clip(m, 0, N_MODULES - 1)
        zm = MODULE_Z[mm]
        x = np.where(alive, x + tx * (zm - zc), x)
        y = np.where(alive, y + ty * (zm - zc), y)
        zc = np.where(alive, zm, zc)
        crossed = alive & _in_acceptance(x, y, MODULE_IS_LEFT[mm])
        seen = crossed & (eff_u[idx, mm] < params.hit_eff)
        if seen.any():
            sel = idx[seen]
            msel = mm[seen]
            out_t.append(sel)
            out_m.append(msel)
            out_x.append(x[seen] + SIGMA_XY * smear[sel, msel, 0])
            out_y.append(y[seen] + SIGMA_XY * smear[sel, msel, 1])
        kick = np.where(crossed, sigma, 0.0)
        tx = tx + kick * ms[idx, mm, 0]
        ty = ty + kick * ms[idx, mm, 1]
    if out_t:
        return (np.concatenate(out_t), np.concatenate(out_m),
                np.concatenate(out_x), np.concatenate(out_y))
    z = np.zeros(0)
    return np.zeros(0, np.int64), np.zeros(0, np.int64), z, z


def _finish_event(rng, params: GenParams, d, t_trk, t_mod, t_x, t_y):
    """Noise hits (drawn after the tracks), module grouping and packing."""
    ntrk = d["p"].shape[0]
    n_real = np.bincount(t_mod, minlength=N_MODULES)
    n_noise = rng.poisson(params.noise_frac * n_real)
    tot_noise = int(n_noise.sum())
    r = np.sqrt(rng.uniform(R_MIN * R_MIN, R_MAX * R_MAX, tot_noise))
    u_phi = rng.uniform(-0.5 * np.pi, 0.5 * np.pi, tot_noise)
    noise_mod = np.repeat(np.arange(N_MODULES), n_noise)
    noise_phi = np.where(MODULE_IS_LEFT[noise_mod], u_phi + np.pi, u_phi)
    n_x = r * np.cos(noise_phi)
    n_y = r * np.sin(noise_phi)

    keys = np.concatenate([t_trk + 1, NOISE_KEY_BASE + np.arange(tot_noise)]).astype(np.uint64)
    mods = np.concatenate([t_mod, noise_mod]).astype(np.int64)
    xs = np.concatenate([t_x, n_x])
    ys = np.concatenate([t_y, n_y])
    order = np.argsort(mods, kind="stable")
    mods = mods[order]
    ids = ((keys[order] << np.uint64(8)) | mods.astype(np.uint64)).astype(np.uint32)
    counts = np.bincount(mods, minlength=N_MODULES).astype(np.int32)
    starts = np.zeros(N_MODULES, np.int32)
    starts[1:] = np.cumsum(counts)[:-1]
    ev = Event(
        sensor_z=np.trunc(MODULE_Z).astype(np.int32),
        hit_start=starts,
        hit_num=counts,
        hit_id=ids,
        x=xs[order].astype(np.float32),
        y=ys[order].astype(np.float32),
        z=MODULE_Z[mods].astype(np.float32),
    )
    truth = Truth(p=d["p"], eta=d["eta"], n_hits=np.bincount(t_trk, minlength=ntrk))
    return ev, truth


def generate_event(seed: int, params: GenParams = CONFIG_SMALL) -> Tuple[Event, Truth]:
    rng = np.random.Generator(np.random.PCG64(seed))
    d = _draw_tracks(rng, params)
    return _finish_event(rng, params, d, *_propagate(d, params))


def generate_events(seeds: Sequence[int], params: GenParams = CONFIG_SMALL):
    """Same events as :func:`generate_event` per seed, propagated as one batch."""
    rngs = [np.random.Generator(np.random.PCG64(int(s))) for s in seeds]
    draws = [_draw_tracks(r, params) for r in rngs]
    if not draws:
        return []
    sizes = np.array([d["p"].shape[0] for d in draws])
    cat = {k: np.concatenate([d[k] for d in draws]) for k in draws[0]}
    t_trk, t_mod, t_x, t_y = _propagate(cat, params)
    bounds = np.concatenate([[0], np.cumsum(sizes)])
    ev_of = np.searchsorted(bounds, t_trk, side="right") - 1
    order = np.argsort(ev_of, kind="stable")
    t_trk, t_mod, t_x, t_y, ev_of = t_trk[order], t_mod[order], t_x[order], t_y[order], ev_of[order]
    cuts = np.searchsorted(ev_of, np.arange(len(draws) + 1))
    out = []
    for i, (r, d) in enumerate(zip(rngs, draws)):
        a, b = cuts[i], cuts[i + 1]
        # the stable sort by event keeps (step, track) order inside an event,
        # which is the order the single-event path records hits in
        tt = t_trk[a:b] - bounds[i]
        mm = t_mod[a:b]
        out.append(_finish_event(r, params, d, tt, mm, t_x[a:b], t_y[a:b]))
    return out


def generate(seeds: Sequence[int], params: GenParams = CONFIG_SMALL):
    """Generate packed blobs (unsorted, file order) and truth for ``seeds``."""
    blobs, truths = [], []
    seeds = list(seeds)
    for i in range(0, len(seeds), 512):
        for ev, tr in generate_events(seeds[i:i + 512], params):
            blobs.append(pack_event(ev))
            truths.append(tr)
    return blobs, truths


def _gen_chunk(args):
    seeds, params = args
    return generate(seeds, params)


def generate_parallel(seeds: Sequence[int], params: GenParams = CONFIG_SMALL, workers: int = 0):
    """:func:`generate` over a ``spawn`` process pool (safe next to CUDA)."""
    import multiprocessing as mp
    import os
    seeds = list(seeds)
    workers = workers or min(len(os.sched_getaffinity(0)), 16)
    if workers <= 1 or len(seeds) < 256:
        return generate(seeds, params)
    chunk = (len(seeds) + workers * 4 - 1) // (workers * 4)
    parts = [(seeds[i:i + chunk], params) for i in range(0, len(seeds), chunk)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        res = pool.map(_gen_chunk, parts)
    blobs, truths = [], []
    for b, t in res:
        blobs.extend(b)
        truths.extend(t)
    return blobs, truths
