"""Learned doublet pruning: training data, training, calibration, evaluation.

The plain method is both the teacher and the yardstick:

* training data -- the search kernel records the features of the doublets that
  reach the h2 search during a plain run (``velo_dump_doublets``, so training
  and in-kernel inference see identical features); a doublet (h0, h1) is
  positive iff an output track starts with h0, h1 (its tracklet survived),
  and its width target is |x predicted at the track's third hit - x of that
  hit|;
* training -- ``velo_mlp_train`` (CUDA forward, backward and Adam kernels,
  batch 4096, lr 1e-3); :func:`reference_loss_and_grad` is the float64 CPU
  restatement its gradients are checked against;
* calibration -- the keep threshold and window margin are set on held-out
  doublets so that nearly every positive keeps its doublet and its h2;
* evaluation -- plain and learned searches of the same held-out events:
  events/s, tracking efficiency, ghost and clone rates, fallback fraction.
"""
from __future__ import annotations

import dataclasses
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import native
from .events import pack_events, unpack_event

N_IN, N_HID, N_OUT = 10, 32, 2
W1, B1 = 0, 320
W2, B2 = 352, 1376
W3, B3 = 1408, 1472
N_PARAMS = 1474
WIDTH_WEIGHT = 0.1


def init_weights(seed: int = 0) -> np.ndarray:
    """He-initialised parameters in the library's flat layout."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = np.zeros(N_PARAMS, np.float32)
    w[W1:B1] = rng.normal(0, np.sqrt(2.0 / N_IN), N_HID * N_IN)
    w[W2:B2] = rng.normal(0, np.sqrt(2.0 / N_HID), N_HID * N_HID)
    w[W3:B3] = rng.normal(0, np.sqrt(1.0 / N_HID), N_OUT * N_HID)
    w[B3 + 1] = 0.2          # start the width near a typical residual
    return w


def unpack(w: np.ndarray):
    w = np.asarray(w, np.float64)
    return (w[W1:B1].reshape(N_HID, N_IN), w[B1:W2], w[W2:B2].reshape(N_HID, N_HID), w[B2:W3],
            w[W3:B3].reshape(N_OUT, N_HID), w[B3:B3 + N_OUT])


def forward_np(w: np.ndarray, x: np.ndarray) -> np.ndarray:
    A, a, B, b, C, c = unpack(w)
    h1 = np.maximum(x @ A.T + a, 0)
    h2 = np.maximum(h1 @ B.T + b, 0)
    return h2 @ C.T + c


def forward_fp16_np(w: np.ndarray, x: np.ndarray) -> np.ndarray:
    """The inference arithmetic of the GPU (velo_mlp_forward, learned seeding):
    features, weights and hidden activations rounded to FP16, sums in FP32
    or wider, biases in FP32."""
    A, a, B, b, C, c = unpack(w)
    h = lambda v: np.asarray(v, np.float32).astype(np.float16).astype(np.float64)
    h1 = np.maximum(h(x) @ h(A).T + a, 0)
    h2 = np.maximum(h(h1) @ h(B).T + b, 0)
    return h(h2) @ h(C).T + c


def reference_loss_and_grad(w: np.ndarray, x: np.ndarray, label: np.ndarray, target: np.ndarray):
    """Mean loss and its gradient in float64 (the CPU check of the CUDA kernels)."""
    A, a, B, b, C, c = unpack(w)
    x = np.asarray(x, np.float64)
    y = np.asarray(label, np.float64)
    t = np.asarray(target, np.float64)
    n = len(x)
    z1 = x @ A.T + a
    h1 = np.maximum(z1, 0)
    z2 = h1 @ B.T + b
    h2 = np.maximum(z2, 0)
    o = h2 @ C.T + c
    z, wd = o[:, 0], o[:, 1]
    bce = np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z)))
    e = wd - t
    loss = np.mean(bce + y * WIDTH_WEIGHT * e * e)
    p = 1 / (1 + np.exp(-z))
    do = np.stack([(p - y) / n, y * 2 * WIDTH_WEIGHT * e / n], axis=1)
    gC = do.T @ h2
    gc = do.sum(0)
    dh2 = (do @ C) * (z2 > 0)
    gB = dh2.T @ h1
    gb = dh2.sum(0)
    dh1 = (dh2 @ B) * (z1 > 0)
    gA = dh1.T @ x
    ga = dh1.sum(0)
    g = np.concatenate([gA.ravel(), ga, gB.ravel(), gb, gC.ravel(), gc])
    return loss, g


@dataclasses.dataclass
class Dataset:
    x: np.ndarray          # (n, 10) float32 features
    label: np.ndarray      # (n,) float32 in {0, 1}
    target: np.ndarray     # (n,) float32 width target (mm), 0 for negatives
    events: int


def build_dataset(ctx: native.Context, blobs: Sequence[bytes], keep_one_in: int = 1,
                  capacity: int = 20_000_000) -> Dataset:
    """Doublets of a plain run over ``blobs`` (x-sorted), labelled by its output."""
    buf, offs, sizes = pack_events(blobs)
    ctx.stage(buf, offs, sizes)
    feats, ids, count = ctx.dump_doublets(capacity, keep_one_in)
    cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs))
    tracks, counts, first, status = ctx.fetch(len(blobs), cap)
    # surviving seeds: per event, h0 -> (h1, h2) from each track's first three hits
    label = np.zeros(len(ids), np.float32)
    target = np.zeros(len(ids), np.float32)
    order = np.argsort(ids[:, 0], kind="stable")
    ev_sorted = ids[order, 0]
    bounds = np.searchsorted(ev_sorted, np.arange(len(blobs) + 1))
    for e in range(len(blobs)):
        rows = order[bounds[e]:bounds[e + 1]]
        if len(rows) == 0 or counts[e] == 0:
            continue
        t = tracks[int(first[e]):int(first[e]) + int(counts[e])]
        seeds = t["hits"][:, :3].astype(np.int64)
        seed_key = (seeds[:, 0] << 32) | seeds[:, 1]       # h0 seeds at most once: keys are unique
        row_key = (ids[rows, 1].astype(np.int64) << 32) | ids[rows, 2].astype(np.int64)
        srt = np.argsort(seed_key)
        pos = np.searchsorted(seed_key[srt], row_key)
        pos = np.minimum(pos, len(srt) - 1)
        hit = seed_key[srt][pos] == row_key
        if not hit.any():
            continue
        r = rows[hit]
        h0, h1, h2 = (seeds[srt][pos[hit], k] for k in range(3))
        ev = unpack_event(blobs[e])
        x0, z0 = ev.x[h0].astype(np.float64), ev.z[h0].astype(np.float64)
        x1, z1 = ev.x[h1].astype(np.float64), ev.z[h1].astype(np.float64)
        xp = x0 + (x1 - x0) * (ev.z[h2].astype(np.float64) - z0) / (z1 - z0)
        label[r] = 1.0
        target[r] = np.abs(xp - ev.x[h2].astype(np.float64))
    return Dataset(feats, label, target, len(blobs))


def train(ds: Dataset, steps: int = 3000, batch: int = 4096, lr: float = 1e-3, seed: int = 0,
          weights: np.ndarray = None) -> Tuple[np.ndarray, np.ndarray]:
    w0 = init_weights(seed) if weights is None else weights
    return native.mlp_train(ds.x, ds.label, ds.target, w0, steps, batch, lr, seed)


def calibrate(w: np.ndarray, ds: Dataset, recall: float = 0.999, width_cover: float = 0.999) -> Tuple[float, float]:
    """Keep threshold and window margin from held-out doublets.

    threshold: the logit below which only (1 - recall) of positives fall;
    margin: added to the predicted width so that width_cover of the kept
    positives have their h2 inside the window."""
    out = native.mlp_forward(w, ds.x)
    pos = ds.label > 0.5
    if not pos.any():
        return -1e30, 10.0
    logits = out[pos, 0]
    thr = float(np.quantile(logits, 1.0 - recall))
    kept = pos & (out[:, 0] >= thr)
    need = ds.target[kept] - np.maximum(out[kept, 1], 0.0)
    margin = float(max(np.quantile(need, width_cover), 0.0)) + 0.01
    return thr, margin


def keep_fraction(w: np.ndarray, ds: Dataset, threshold: float) -> float:
    out = native.mlp_forward(w, ds.x)
    return float(np.mean(out[:, 0] >= threshold))


def evaluate(ctx: native.Context, blobs: Sequence[bytes], truths, base: native.Options = None,
             iters: int = 5) -> Dict[str, Dict]:
    """Plain vs learned on the same events (weights already set on ``ctx``)."""
    from .validation import rates
    base = base or native.default_options()
    res = {}
    for name, learned in (("plain", 0), ("learned", 1)):
        o = native.Options.from_buffer_copy(base)
        o.learned = learned
        buf, offs, sizes = pack_events(blobs)
        ctx.stage(buf, offs, sizes)
        ctx.run(o)
        cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs))
        tracks, counts, first, status = ctx.fetch(len(blobs), cap)
        per = [tracks[int(first[e]):int(first[e]) + int(counts[e])] for e in range(len(blobs))]
        ms = sorted(ctx.time_runs(o, warmup=1, iters=1, flush_l2=True) for _ in range(iters))[iters // 2]
        r = rates(per, blobs, truths)
        res[name] = dict(r.as_dict(), ms=ms, events_per_s=len(blobs) / (ms / 1e3),
                         fallback=int(np.sum((status & native.EVENT_LEARNED_FALLBACK) != 0)),
                         tracks_list=per)
    return res


# --------------------------------------------------------------- driver --
def _sorted_events(seeds, params):
    from .generator import generate_parallel
    raw, truths = generate_parallel(seeds, params)
    return [native.sort_by_x(b) for b in raw], truths


def _chunks(n, size):
    return [(a, min(n, a + size)) for a in range(0, n, size)]


def compare_paths(ctx, blobs, truths, weights, thr, margin, min_keep, options, chunk=10000, iters=3, max_hits=0):
    """Plain vs learned over ``blobs`` in chunks: events/s (device time), rates, fallbacks."""
    from .validation import Rates, rates_fast
    out = {}
    for name, learned_flag in (("plain", 0), ("learned", 1)):
        o = native.Options.from_buffer_copy(options)
        o.learned = learned_flag
        total_ms, r, fb = 0.0, Rates(), 0
        for a, b in _chunks(len(blobs), chunk):
            sub = blobs[a:b]
            buf, offs, sizes = pack_events(sub)
            ctx.stage(buf, offs, sizes)
            if learned_flag:
                ctx.set_mlp(weights, thr, margin, min_keep, max_hits)
            ms = sorted(ctx.time_runs(o, warmup=1 if i == 0 else 0, iters=1, flush_l2=True) for i in range(iters))
            total_ms += ms[len(ms) // 2]
            ctx.run(o)
            cap = int(sum(max(int(np.frombuffer(x[4:8], "<i4")[0]), 1) for x in sub))
            tracks, counts, first, status = ctx.fetch(len(sub), cap)
            per = [tracks[int(first[e]):int(first[e]) + int(counts[e])] for e in range(len(sub))]
            r.add(rates_fast(per, sub, truths[a:b]))
            fb += int(np.sum((status & native.EVENT_LEARNED_FALLBACK) != 0))
        out[name] = dict(r.as_dict(), ms=total_ms, events_per_s=len(blobs) / (total_ms / 1e3), fallback=fb,
                         fallback_fraction=fb / max(len(blobs), 1))
    p, l = out["plain"], out["learned"]
    out["delta"] = {"efficiency_loss": p["efficiency"] - l["efficiency"],
                    "ghost_increase": l["ghost_rate"] - p["ghost_rate"],
                    "clone_change": l["clone_rate"] - p["clone_rate"],
                    "speedup": l["events_per_s"] / p["events_per_s"]}
    return out


def main(argv=None):
    import argparse
    import hashlib
    import json
    import os
    import time
    from . import generator
    ap = argparse.ArgumentParser(description="train and evaluate the learned doublet pruning")
    ap.add_argument("--train-events", type=int, default=50000)
    ap.add_argument("--heldout-events", type=int, default=10000)
    ap.add_argument("--calib-events", type=int, default=1000)
    ap.add_argument("--stress-events", type=int, default=100000)
    ap.add_argument("--keep-one-in", type=int, default=50, help="training doublets sampled 1 in N")
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--recall", type=float, default=0.999)
    ap.add_argument("--min-keep-rate", type=float, default=0.02)
    ap.add_argument("--max-hits-factor", type=float, default=1.0,
                    help="events above this x the largest training event take the plain method")
    ap.add_argument("--out", default="learned_out")
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    t0 = time.time()
    # event generation first (process pool before any GPU work)
    train_blobs, _ = _sorted_events(range(100000, 100000 + a.train_events), generator.CONFIG_SMALL)
    calib_blobs, _ = _sorted_events(range(1010000, 1010000 + a.calib_events), generator.CONFIG_SMALL)
    held_blobs, held_truths = _sorted_events(range(1000000, 1000000 + a.heldout_events), generator.CONFIG_SMALL)
    print(f"generated {len(train_blobs)}+{len(calib_blobs)}+{len(held_blobs)} events in {time.time() - t0:.0f}s",
          flush=True)
    ctx = native.Context(0)
    parts = []
    for lo, hi in _chunks(len(train_blobs), 10000):
        parts.append(build_dataset(ctx, train_blobs[lo:hi], keep_one_in=a.keep_one_in, capacity=4_000_000))
    train_hits = np.array([int(np.frombuffer(b[4:8], "<i4")[0]) for b in train_blobs])
    max_hits = int(a.max_hits_factor * train_hits.max())
    ds = Dataset(np.concatenate([p.x for p in parts]), np.concatenate([p.label for p in parts]),
                 np.concatenate([p.target for p in parts]), len(train_blobs))
    cal = build_dataset(ctx, calib_blobs, keep_one_in=1, capacity=20_000_000)
    print(f"training doublets {len(ds.x)} ({int(ds.label.sum())} positive); calibration {len(cal.x)}", flush=True)
    t1 = time.time()
    w, losses = train(ds, steps=a.steps, batch=4096, lr=1e-3, seed=0)
    train_s = time.time() - t1
    thr, margin = calibrate(w, cal, recall=a.recall)
    kept = keep_fraction(w, cal, thr)
    w0 = init_weights(0)
    thr0, _ = calibrate(w0, cal, recall=a.recall)
    kept0 = keep_fraction(w0, cal, thr0)
    base = native.default_options(launch_mode=1, threads_per_event=64, smem_hits=50, register_ctas=4)
    res4 = compare_paths(ctx, held_blobs, held_truths, w, thr, margin, a.min_keep_rate, base, max_hits=max_hits)
    report = {"config4": {"train_events": len(train_blobs), "train_doublets": int(len(ds.x)),
                          "train_positive": int(ds.label.sum()), "steps": a.steps, "batch": 4096, "lr": 1e-3,
                          "train_seconds": train_s, "loss_first": float(losses[:50].mean()),
                          "loss_last": float(losses[-50:].mean()), "keep_threshold": thr, "window_margin": margin,
                          "kept_fraction": kept, "kept_fraction_untrained": kept0,
                          "max_event_hits": max_hits, "train_hits_mean": float(train_hits.mean()),
                          "heldout_events": len(held_blobs), "results": res4}}
    print(json.dumps(report["config4"]["results"]["delta"]), flush=True)
    np.savez(os.path.join(a.out, "doublet_mlp.npz"), weights=w, keep_threshold=np.float32(thr),
             window_margin=np.float32(margin), min_keep_rate=np.float32(a.min_keep_rate),
             max_event_hits=np.uint32(max_hits), sha256=hashlib.sha256(w.tobytes()).hexdigest())
    del train_blobs, ds
    if a.stress_events:
        sb, st = _sorted_events(range(3000000, 3000000 + a.stress_events), generator.CONFIG_STRESS)
        res5 = compare_paths(ctx, sb, st, w, thr, margin, a.min_keep_rate, base, max_hits=max_hits)
        res5_open = compare_paths(ctx, sb, st, w, thr, margin, a.min_keep_rate, base, max_hits=0)
        report["config5"] = {"events": len(sb), "mean_hits": float(np.mean([int(np.frombuffer(b[4:8], "<i4")[0])
                                                                             for b in sb])), "results": res5,
                             "results_without_hits_guard": res5_open}
        print(json.dumps(res5["delta"]), json.dumps(res5_open["delta"]), flush=True)
    with open(os.path.join(a.out, "learned_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    print(f"done in {time.time() - t0:.0f}s", flush=True)


if __name__ == "__main__":
    main()
