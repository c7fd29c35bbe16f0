"""velo_search_device_static: the search for callers that cannot allocate.

Some callers cannot call cudaMalloc: code under a framework that owns every
device allocation, or a path that must keep a fixed device footprint.  This
entry point takes device buffers for the events and the results and keeps
all of its own working memory in one fixed file-scope device array.  Its
results must equal those of the allocating entry point (velo_search), exactly,
on consecutive calls that reuse the shared array.

This file is collected last (test_zz_*), so a stop-at-first-failure run has
run every other test before it; it also passes on its own in a fresh process.
Device buffers for the caller's side come from torch, used as a plain
allocator here.
"""
import numpy as np
import pytest

from conftest import index_lists

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _hits(blob):
    return int(np.frombuffer(blob[4:8], "<i4")[0])


def _call_static(lib, blobs, y=4, max_event_hits=None, total_hits=None, capacity=None):
    from cl_forward_gb300 import events
    n = len(blobs)
    buf, offs, sizes = events.pack_events(blobs)
    H = [_hits(b) for b in blobs]
    total = sum(H) if total_hits is None else total_hits
    maxh = max(H) if max_event_hits is None else max_event_hits
    cap = total + n if capacity is None else capacity
    d_buf = torch.from_numpy(buf).cuda()
    d_offs = torch.from_numpy(offs.astype(np.int64)).cuda()
    d_sizes = torch.from_numpy(sizes.astype(np.int64)).cuda()
    d_tracks = torch.zeros(max(cap, 1) * 25, dtype=torch.int32, device="cuda")
    d_counts = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    d_first = torch.zeros(max(n, 1), dtype=torch.int64, device="cuda")
    d_status = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.velo_search_device_static(d_buf.data_ptr(), d_offs.data_ptr(), d_sizes.data_ptr(), n, total, maxh, y,
                                       d_tracks.data_ptr(), cap, d_counts.data_ptr(), d_first.data_ptr(),
                                       d_status.data_ptr(), stream)
    torch.cuda.synchronize()
    if st != 0:
        return st, None, None
    tracks = d_tracks.cpu().numpy().view(np.uint32).reshape(-1, 25)
    counts = d_counts.cpu().numpy().view(np.uint32)[:n]
    first = d_first.cpu().numpy().view(np.uint64)[:n]
    status = d_status.cpu().numpy().view(np.uint32)[:n]
    per_event = [tracks[int(first[e]):int(first[e]) + int(counts[e])] for e in range(n)]
    return 0, per_event, status


def _lists(words):
    return sorted(tuple(int(h) for h in w[1:1 + int(w[0])]) for w in words)


@pytest.fixture(scope="module")
def lib_and_ctx():
    from cl_forward_gb300 import build, native
    build.build()
    lib = native.load()
    ctx = native.Context(0)
    yield lib, ctx
    ctx.close()


def test_static_matches_allocating_entry_point_on_consecutive_calls(lib_and_ctx):
    from cl_forward_gb300 import fuzz, generator, native
    lib, ctx = lib_and_ctx
    batch_a = [native.sort_by_x(b) for b in generator.generate(range(30))[0]]
    # denser events, within the entry point's per-event limit (10,676 hits)
    dense = generator.generate(range(50, 90), generator.CONFIG_BATCHED)[0]
    batch_b = [native.sort_by_x(b) for b in dense if _hits(b) <= 3200]
    assert len(batch_b) >= 5
    batch_b += [native.sort_by_x(fuzz.fuzz_event(5000 + s, max_per_module=20, grid=1.0, lines=10, x_span=45))
                for s in range(10)]
    for batch in (batch_a, batch_b, batch_a):      # the third call sees the second call's leftovers
        st, got, status = _call_static(lib, batch)
        assert st == 0
        want, want_status = ctx.search(batch, native.default_options())
        assert np.array_equal(status, want_status)
        for e in range(len(batch)):
            assert _lists(got[e]) == index_lists(want[e]), f"event {e}"
            # whole records, as the allocating path writes them
            assert sorted(map(tuple, got[e].tolist())) == \
                sorted(map(tuple, want[e].view(np.uint32).reshape(-1, 25).tolist()))


def test_static_y_lanes(lib_and_ctx):
    from cl_forward_gb300 import fuzz, native
    lib, ctx = lib_and_ctx
    batch = [native.sort_by_x(fuzz.fuzz_event(5100 + s, max_per_module=20, grid=1.0, lines=10, x_span=45))
             for s in range(20)]
    for y in (1, 3):
        st, got, _ = _call_static(lib, batch, y=y)
        assert st == 0
        want, _ = ctx.search(batch, native.default_options(y_lanes=y))
        assert [_lists(g) for g in got] == [index_lists(w) for w in want]


def test_static_limits_are_rejected(lib_and_ctx):
    from cl_forward_gb300 import generator, native
    lib, _ = lib_and_ctx
    batch = [native.sort_by_x(b) for b in generator.generate(range(3))[0]]
    total = sum(_hits(b) for b in batch)
    assert _call_static(lib, batch, total_hits=native.STATIC_MAX_HIT_ROWS)[0] == native.ERR_CAPACITY
    assert _call_static(lib, batch, capacity=total)[0] == native.ERR_CAPACITY
    assert _call_static(lib, batch, max_event_hits=100000)[0] == native.ERR_CAPACITY
    assert _call_static(lib, batch, y=17)[0] == native.ERR_INVALID_ARGUMENT
    st = lib.velo_search_device_static(None, None, None, native.STATIC_MAX_EVENTS + 1, 0, 100, 4, None, 0,
                                       None, None, None, None)
    assert st == native.ERR_CAPACITY


def test_static_event_over_its_declared_bound_is_invalid(lib_and_ctx):
    from cl_forward_gb300 import generator, native
    lib, ctx = lib_and_ctx
    batch = [native.sort_by_x(b) for b in generator.generate(range(100, 106))[0]]
    H = [_hits(b) for b in batch]
    bound = max(H) - 1                         # the largest event breaks its declared bound
    over = [e for e in range(len(batch)) if H[e] > bound]
    st, got, status = _call_static(lib, batch, max_event_hits=bound)
    assert st == 0
    want, _ = ctx.search(batch, native.default_options())
    for e in range(len(batch)):
        if e in over:
            assert status[e] & native.EVENT_INVALID and len(got[e]) == 0
        else:
            assert _lists(got[e]) == index_lists(want[e])
