"""Autotuner cache logic (the sweep itself runs on the GPU, in test_gpu_parity)."""
from cl_forward_gb300 import autotune


class FakeOptions:
    def __init__(self, **kw):
        self.y_lanes = 4
        self.threads_per_event = 256
        self.launch_mode = 0
        self.smem_hits = 0
        self.narrow_windows = 1
        self.register_ctas = 5
        self.seed_lanes = 32
        self.__dict__.update(kw)


class FakeCtx:
    sm_count = 152

    def __init__(self):
        self.calls = 0

    def autotune(self, base, iters):
        self.calls += 1
        return FakeOptions(threads_per_event=128, launch_mode=1, smem_hits=900, register_ctas=4, seed_lanes=8), 5.5


def test_shape_key_buckets():
    assert autotune.shape_key(152, 10000, 1161, 4) == autotune.shape_key(152, 9000, 1100, 4)
    assert autotune.shape_key(152, 10000, 1161, 4) != autotune.shape_key(152, 10000, 3000, 4)
    assert autotune.shape_key(152, 10000, 1161, 4) != autotune.shape_key(152, 10000, 1161, 1)


def test_tune_once_then_cached(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune.native, "default_options", lambda: FakeOptions())
    path = str(tmp_path / "cache.json")
    ctx = FakeCtx()
    o1, info1 = autotune.tuned_options(ctx, 10000, 1161, iters=2, cache_path=path)
    o2, info2 = autotune.tuned_options(ctx, 10000, 1161, iters=2, cache_path=path)
    assert ctx.calls == 1 and not info1["cached"] and info2["cached"]
    for o in (o1, o2):
        assert (o.threads_per_event, o.launch_mode, o.smem_hits, o.register_ctas, o.seed_lanes) == (128, 1, 900, 4, 8)
    autotune.tuned_options(ctx, 10000, 1161, iters=2, cache_path=path, refresh=True)
    assert ctx.calls == 2
