"""The learned doublet pruning on the GPU: kernels, data, and what it gains.

The CUDA forward / backward / Adam kernels are checked against the float64
CPU restatement; the dump of training doublets against the plain output; the
learned seeding with nothing pruned against the plain seeding (identical
tracks); and a trained network against an untrained one on held-out events
(same recall target: the trained one prunes far more doublets, within the
efficiency and ghost budgets).
"""
import numpy as np
import pytest

from conftest import index_lists

pytestmark = pytest.mark.gpu


def _data(n, seed):
    from cl_forward_gb300 import learned
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.normal(0, 1, (n, learned.N_IN)).astype(np.float32)
    y = (rng.random(n) < 0.2).astype(np.float32)
    t = (np.abs(rng.normal(0.1, 0.05, n)) * y).astype(np.float32)
    return x, y, t


def test_mlp_gradients_match_cpu(native_lib):
    from cl_forward_gb300 import learned, native
    w = learned.init_weights(5)
    x, y, t = _data(3000, 7)
    g, loss = native.mlp_grad(w, x, y, t)
    loss_ref, g_ref = learned.reference_loss_and_grad(w, x, y, t)
    assert abs(loss - loss_ref) <= 1e-5 * max(1.0, abs(loss_ref))
    scale = np.abs(g_ref).max()
    assert np.max(np.abs(g - g_ref)) <= 2e-4 * scale + 1e-7

def test_mlp_inference_matches_fp16_restatement(native_lib):
    """Tensor-core inference (FP16 operands, FP32 sums) against the same
    rounding done in numpy, and within FP16 error of the FP32 network.  The
    tolerance allows one FP16 rounding of a hidden unit to land on the other
    side (2^-11 relative) through the following layers."""
    from cl_forward_gb300 import learned, native
    for seed in (5, 6):
        w = learned.init_weights(seed)
        x, _, _ = _data(5001, seed)          # a partial last warp
        out = native.mlp_forward(w, x)
        ref16 = learned.forward_fp16_np(w, x)
        scale = 1.0 + np.abs(ref16)
        assert np.max(np.abs(out - ref16) / scale) < 2e-3
        assert np.max(np.abs(out - learned.forward_np(w, x)) / scale) < 3e-2


def test_training_reduces_loss(native_lib):
    from cl_forward_gb300 import learned, native
    rng = np.random.Generator(np.random.PCG64(2))
    x = rng.normal(0, 1, (20000, learned.N_IN)).astype(np.float32)
    y = (x[:, 0] + 0.5 * x[:, 3] > 0.3).astype(np.float32)           # learnable rule
    t = (0.05 + 0.02 * np.abs(x[:, 1]) * y).astype(np.float32)
    w, losses = native.mlp_train(x, y, t, learned.init_weights(1), steps=400, batch=4096, lr=1e-3, seed=3)
    assert losses[-20:].mean() < 0.5 * losses[:20].mean()
    acc = np.mean((native.mlp_forward(w, x)[:, 0] > 0) == (y > 0.5))
    assert acc > 0.95


def test_dump_labels_match_output(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator, learned
    blobs = [oracle_lib.sort_by_x(b) for b in generator.generate(range(100000, 100030))[0]]
    ds = learned.build_dataset(gpu_ctx, blobs)
    assert len(ds.x) > 1000 and np.isfinite(ds.x).all()
    want, _ = oracle_lib.search(blobs, 4)
    # every output track's seed doublet reached the h2 search, so it was recorded
    assert int(ds.label.sum()) == sum(len(t) for t in want)
    assert np.all(ds.target[ds.label > 0] < 0.6) and np.all(ds.target[ds.label == 0] == 0)


def test_learned_with_nothing_pruned_equals_plain(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator, learned, native
    blobs = [oracle_lib.sort_by_x(b) for b in generator.generate(range(100100, 100140))[0]]
    gpu_ctx.set_mlp(learned.init_weights(0), keep_threshold=-1e30, window_margin=100.0, min_keep_rate=0.0)
    got, status = gpu_ctx.search(blobs, native.default_options(learned=1))
    want, _ = oracle_lib.search(blobs, 4)
    assert not np.any(status & native.EVENT_LEARNED_FALLBACK)
    for e in range(len(blobs)):
        assert index_lists(got[e]) == index_lists(want[e])
    # an impossible keep rate sends every event back to the plain search: same tracks, flagged
    gpu_ctx.set_mlp(learned.init_weights(0), keep_threshold=1e30, window_margin=0.0, min_keep_rate=0.5)
    got, status = gpu_ctx.search(blobs, native.default_options(learned=1))
    assert np.all(status & native.EVENT_LEARNED_FALLBACK)
    for e in range(len(blobs)):
        assert index_lists(got[e]) == index_lists(want[e])
    # events above the hit-count limit take the plain method from the start
    hits = np.array([int(np.frombuffer(b[4:8], "<i4")[0]) for b in blobs])
    limit = int(np.median(hits))
    gpu_ctx.set_mlp(learned.init_weights(0), keep_threshold=1e30, window_margin=0.0, min_keep_rate=0.0,
                    max_event_hits=limit)
    got, status = gpu_ctx.search(blobs, native.default_options(learned=1))
    over = hits > limit
    assert over.any() and (~over).any()
    assert np.array_equal((status & native.EVENT_LEARNED_FALLBACK) != 0, over)
    for e in np.flatnonzero(over):
        assert index_lists(got[e]) == index_lists(want[e])
    for e in np.flatnonzero(~over):          # everything pruned: no seeds, no tracks
        assert len(got[e]) == 0


@pytest.mark.parametrize("lanes", [8, 32])
def test_learned_gate_above_every_window_scores_nothing(gpu_ctx, oracle_lib, lanes):
    """learned_min_window: doublets whose exact h2 window holds fewer hits
    than the gate are searched exactly, unscored.  With a network that would
    prune everything (keep threshold above any logit) and a gate above every
    window, nothing is scored, so the tracks are the plain method's and no
    event falls back (the keep-rate guard counts scored doublets only); at a
    gate of 0 the same network prunes every doublet and every event falls
    back to the plain search."""
    from cl_forward_gb300 import generator, learned, native
    blobs = [oracle_lib.sort_by_x(b) for b in generator.generate(range(100200, 100230))[0]]
    want, _ = oracle_lib.search(blobs, 4)
    gpu_ctx.set_mlp(learned.init_weights(0), keep_threshold=1e30, window_margin=0.0, min_keep_rate=0.5)
    got, status = gpu_ctx.search(blobs, native.default_options(learned=1, learned_min_window=1 << 20,
                                                               seed_lanes=lanes))
    assert not np.any(status & native.EVENT_LEARNED_FALLBACK)
    assert [index_lists(g) for g in got] == [index_lists(w) for w in want]
    got, status = gpu_ctx.search(blobs, native.default_options(learned=1, learned_min_window=0, seed_lanes=lanes))
    assert np.all(status & native.EVENT_LEARNED_FALLBACK)
    assert [index_lists(g) for g in got] == [index_lists(w) for w in want]
    with pytest.raises(native.VeloError):
        gpu_ctx.search(blobs, native.default_options(learned=1, learned_min_window=-1))


def test_trained_network_gains_over_untrained(gpu_ctx, oracle_lib):
    """Same recall target on held-out doublets: the trained scorer prunes much
    more, and the pruned search stays within 0.5 % efficiency and 0.2 % ghost
    rate of the plain search on held-out events."""
    from cl_forward_gb300 import generator, learned, native
    train = [oracle_lib.sort_by_x(b) for b in generator.generate(range(100000, 100300), generator.CONFIG_SMALL)[0]]
    calib = [oracle_lib.sort_by_x(b) for b in generator.generate(range(1000000, 1000100))[0]]
    held, truths = generator.generate(range(1000100, 1000500))
    held = [oracle_lib.sort_by_x(b) for b in held]
    ds = learned.build_dataset(gpu_ctx, train)
    cal = learned.build_dataset(gpu_ctx, calib)
    w, losses = learned.train(ds, steps=1500, seed=0)
    assert losses[-50:].mean() < losses[:50].mean()
    w0 = learned.init_weights(0)
    thr, margin = learned.calibrate(w, cal, recall=0.999)
    thr0, _ = learned.calibrate(w0, cal, recall=0.999)
    kept_trained = learned.keep_fraction(w, cal, thr)
    kept_random = learned.keep_fraction(w0, cal, thr0)
    assert kept_trained < kept_random - 0.1, (kept_trained, kept_random)
    gpu_ctx.set_mlp(w, thr, margin, min_keep_rate=0.02)
    res = learned.evaluate(gpu_ctx, held, truths)
    p, l = res["plain"], res["learned"]
    assert p["efficiency"] - l["efficiency"] <= 0.005
    assert l["ghost_rate"] - p["ghost_rate"] <= 0.002
    print(f"kept {kept_trained:.3f} (untrained {kept_random:.3f}); plain {p['events_per_s']:.0f} ev/s "
          f"eff {p['efficiency']:.4f} ghost {p['ghost_rate']:.4f}; learned {l['events_per_s']:.0f} ev/s "
          f"eff {l['efficiency']:.4f} ghost {l['ghost_rate']:.4f} fallback {l['fallback']}")


def test_learned_through_streamed_and_sorting_paths(gpu_ctx, oracle_lib):
    """The learned kernel shares the staging, the in-kernel sort and the
    streamed records with the plain one: velo_search_begin (with and without
    the sort) and velo_sort_search give the tracks of the synchronous learned
    search of the pre-sorted events, event by event."""
    import os
    import time
    from cl_forward_gb300 import generator, native
    wz = np.load(os.path.join(os.path.dirname(__file__), "..", "cl_forward_gb300", "weights", "doublet_mlp.npz"))
    gpu_ctx.set_mlp(wz["weights"], float(wz["keep_threshold"]), float(wz["window_margin"]),
                    float(wz["min_keep_rate"]), int(wz["max_event_hits"]))
    raw = generator.generate(range(100300, 100360))[0]
    srt = [oracle_lib.sort_by_x(b) for b in raw]
    o = native.default_options(learned=1, host_direct=1)
    want, wst = gpu_ctx.search(srt, o)
    for sort, src in ((0, srt), (1, raw)):
        bufs = [bytearray(b) for b in src]
        results, tracks, keep = gpu_ctx.search_begin(bufs, sort=bool(sort), options=o)
        t0 = time.perf_counter()
        while not results["ready"].all():
            assert time.perf_counter() - t0 < 60
            time.sleep(0.0005)
        counts, first, status = gpu_ctx.search_end(len(bufs))
        assert [bytes(b) for b in bufs] == srt
        assert np.array_equal(status, wst)
        for e in range(len(src)):
            got = tracks[int(first[e]):int(first[e]) + int(counts[e])]
            assert index_lists(got) == index_lists(want[e]), (sort, e)
        del keep
    bufs = [bytearray(b) for b in raw]
    got, status = gpu_ctx.sort_search(bufs, o)
    assert [bytes(b) for b in bufs] == srt and np.array_equal(status, wst)
    assert [index_lists(g) for g in got] == [index_lists(w) for w in want]
