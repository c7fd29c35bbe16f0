"""Parity of the sm_103a search with the reference, through the C ABI.

Golden vectors are the reference kernel's own outputs; everything else is
compared against the oracle restatement (pinned to the reference by
test_golden_oracle.py / test_oracle_vs_reference.py) on the same seeded
events.  Results are integer hit-index lists: the bar is exact equality of
the per-event track multisets.  Events on which the reference itself is
undefined (ring / track-size / track-count overflow) are excluded from
equality and checked for matching status bits instead.
"""
import numpy as np
import pytest

from conftest import GOLDEN_SETS, GOLDEN_Y, index_lists, index_lists_words

pytestmark = pytest.mark.gpu

OVERFLOW_BITS = 0x1 | 0x2 | 0x4


def _sorted(oracle_lib, blobs):
    return [oracle_lib.sort_by_x(b) for b in blobs]


def _assert_same(gpu_ctx, oracle_lib, blobs, y=4, **opts):
    from cl_forward_gb300 import native
    got, gst = gpu_ctx.search(blobs, native.default_options(y_lanes=y, **opts))
    want, ost = oracle_lib.search(blobs, y)
    assert np.array_equal(gst & OVERFLOW_BITS, ost & OVERFLOW_BITS)
    checked = 0
    for e in range(len(blobs)):
        if ost[e] & oracle_lib.PARITY_EXCLUDING:
            continue
        assert index_lists(got[e]) == index_lists(want[e]), f"event {e} differs (opts {opts}, Y={y})"
        checked += 1
    return got, checked


@pytest.mark.parametrize("lanes", [8, 16, 32])
@pytest.mark.parametrize("name", GOLDEN_SETS)
@pytest.mark.parametrize("y", GOLDEN_Y)
def test_golden_vectors(gpu_ctx, golden, name, y, lanes):
    """The reference kernel's own outputs, with every seeding width (lanes per h0)."""
    from cl_forward_gb300 import native
    got, status = gpu_ctx.search(golden[name]["sorted"], native.default_options(y_lanes=y, seed_lanes=lanes))
    assert not np.any(status)
    for e, ref in enumerate(golden[name]["tracks"][y]):
        assert index_lists(got[e]) == index_lists_words(ref), f"{name} event {e}"
        # whole 100-byte records, zero beyond hitsNum, as the reference writes them
        words = got[e].view(np.uint32).reshape(-1, 25)
        assert sorted(map(tuple, words.tolist())) == sorted(map(tuple, ref.tolist()))


def test_config_small_100_events(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator
    blobs = _sorted(oracle_lib, generator.generate(range(100))[0])
    _, n = _assert_same(gpu_ctx, oracle_lib, blobs)
    assert n == 100


@pytest.mark.parametrize("y,lanes", [(1, 8), (1, 32), (2, 16), (3, 32), (4, 8), (4, 16), (4, 32), (8, 8),
                                     (16, 16), (16, 32)])
def test_fuzz_ties_and_lanes(gpu_ctx, oracle_lib, y, lanes):
    """Exact fit ties and wide h1 windows: the winner's (fit, Y-lane, h1, h2)
    order and each Y-lane's stop at its first h1 without an h2 window must
    hold whether one h0's candidates span one warp or a group of 8 or 16
    lanes (several chunks per group, Y-lanes that do or do not divide 32)."""
    from cl_forward_gb300 import fuzz
    blobs = [fuzz.fuzz_event(5000 + s, max_per_module=20, grid=1.0, lines=10, x_span=45) for s in range(150)]
    blobs += [fuzz.fuzz_event(2000 + s, jitter_z=True) for s in range(50)]
    blobs += [fuzz.fuzz_event(s, grid=2.0) for s in range(50)]
    blobs += [fuzz.fuzz_event(3000 + s, n_modules=3 + s % 20) for s in range(40)]
    blobs += [fuzz.fuzz_event(7000 + s, max_per_module=60, grid=0.5, lines=30, x_span=20) for s in range(40)]
    _, n = _assert_same(gpu_ctx, oracle_lib, _sorted(oracle_lib, blobs), y=y, seed_lanes=lanes)
    assert n > 200


@pytest.mark.parametrize("y,lanes", [(4, 12), (4, 64), (3, 8), (3, 16), (8, 4), (16, 8)])
def test_seed_lanes_rejected(gpu_ctx, oracle_lib, y, lanes):
    """Seeding widths other than 8, 16 and 32, or below 32 and not a multiple of Y."""
    from cl_forward_gb300 import generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(2))[0])
    with pytest.raises(native.VeloError) as err:
        gpu_ctx.search(blobs, native.default_options(y_lanes=y, seed_lanes=lanes))
    assert err.value.status == native.ERR_INVALID_ARGUMENT
    got, _ = gpu_ctx.search(blobs, native.default_options(y_lanes=y))   # automatic width
    want, _ = oracle_lib.search(blobs, y)
    assert [index_lists(g) for g in got] == [index_lists(w) for w in want]


@pytest.mark.parametrize("threads", [32, 64, 128, 256, 512])
@pytest.mark.parametrize("mode", [0, 1])
def test_launch_shapes(gpu_ctx, oracle_lib, threads, mode):
    from cl_forward_gb300 import generator
    blobs = _sorted(oracle_lib, generator.generate(range(500, 540))[0])
    _assert_same(gpu_ctx, oracle_lib, blobs, threads_per_event=threads, launch_mode=mode)


@pytest.mark.parametrize("narrow", [0, 1])
@pytest.mark.parametrize("smem_hits", [0, 200])
def test_narrowing_and_global_arena(gpu_ctx, oracle_lib, narrow, smem_hits):
    """smem_hits=200 sends most events to the global-memory arena."""
    from cl_forward_gb300 import fuzz, generator
    blobs = generator.generate(range(600, 630))[0]
    blobs += [fuzz.fuzz_event(2100 + s, jitter_z=True) for s in range(20)]
    blobs = _sorted(oracle_lib, blobs)
    _assert_same(gpu_ctx, oracle_lib, blobs, narrow_windows=narrow, smem_hits=smem_hits)
    assert smem_hits == 0 or gpu_ctx.stats().events_in_global > 0


def test_register_builds_and_graph_replay(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator
    blobs = _sorted(oracle_lib, generator.generate(range(650, 680))[0])
    for regs in (4, 5):
        _assert_same(gpu_ctx, oracle_lib, blobs, register_ctas=regs)
        _assert_same(gpu_ctx, oracle_lib, blobs, register_ctas=regs, use_graph=1, launch_mode=1)
    # the 56-register 64-thread build, one CTA per event and persistent, with and without a tile
    for mode in (0, 1):
        for hits in (0, 50):
            _assert_same(gpu_ctx, oracle_lib, blobs, register_ctas=18, threads_per_event=64, launch_mode=mode,
                         smem_hits=hits)
    from cl_forward_gb300 import native
    with pytest.raises(native.VeloError):                   # the 64-thread build takes 64 threads only
        gpu_ctx.search(blobs, native.default_options(register_ctas=18, threads_per_event=128))


def test_graph_replays_on_staged_events(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import events, generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(950, 990))[0])
    want, _ = oracle_lib.search(blobs, 4)
    buf, offs, sizes = events.pack_events(blobs)
    cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs))
    gpu_ctx.stage(buf, offs, sizes)
    o = native.default_options(use_graph=1)
    for _ in range(3):                                   # capture once, replay
        gpu_ctx.run(o)
        tracks, counts, first, _ = gpu_ctx.fetch(len(blobs), cap)
        for e in range(len(blobs)):
            assert index_lists(tracks[int(first[e]):int(first[e]) + int(counts[e])]) == index_lists(want[e])
    assert gpu_ctx.time_runs(o, warmup=1, iters=2) > 0


def test_autotuned_options_keep_parity(gpu_ctx, oracle_lib, tmp_path):
    from cl_forward_gb300 import autotune, events, generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(1500, 1700))[0])
    buf, offs, sizes = events.pack_events(blobs)
    gpu_ctx.stage(buf, offs, sizes)
    o, info = autotune.tuned_options(gpu_ctx, len(blobs), 1100.0, iters=2, cache_path=str(tmp_path / "c.json"))
    assert info["ms"] > 0 and o.register_ctas in (4, 5)
    _assert_same(gpu_ctx, oracle_lib, blobs, **{k: getattr(o, k) for k in autotune.FIELDS})


def test_unsorted_input_takes_exact_scans(gpu_ctx, oracle_lib):
    """Without the x-sort the reference's window scans still define the output."""
    from cl_forward_gb300 import generator
    blobs = generator.generate(range(700, 720))[0]            # file order, not sorted
    _assert_same(gpu_ctx, oracle_lib, blobs)


def test_dense_and_uneven_events(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator
    blobs = generator.generate(range(100), generator.CONFIG_STRESS)[0]
    blobs += generator.generate(range(200), generator.CONFIG_BATCHED)[0]
    blobs = _sorted(oracle_lib, blobs)
    for mode in (0, 1):
        _, n = _assert_same(gpu_ctx, oracle_lib, blobs, launch_mode=mode)
        assert n > 250


def test_config_scale_10000_events(gpu_ctx, oracle_lib):
    """10,000 events (seeds 1000..10999): set parity and identical tracking rates."""
    from cl_forward_gb300 import generator, native, validation
    raw, truths = generator.generate_parallel(range(1000, 11000))
    blobs = _sorted(oracle_lib, raw)
    got, gst = gpu_ctx.search(blobs, native.default_options())
    want, ost = oracle_lib.search(blobs, 4)
    assert np.array_equal(gst & OVERFLOW_BITS, ost & OVERFLOW_BITS)
    keep = [e for e in range(len(blobs)) if not (ost[e] & oracle_lib.PARITY_EXCLUDING)]
    assert len(keep) > 9900
    bad = [e for e in keep if index_lists(got[e]) != index_lists(want[e])]
    assert not bad, bad[:10]
    rg = validation.rates(got, blobs, truths)
    ro = validation.rates(want, blobs, truths)
    assert abs(rg.efficiency - ro.efficiency) <= 1e-3
    assert abs(rg.ghost_rate - ro.ghost_rate) <= 1e-3
    assert abs(rg.clone_rate - ro.clone_rate) <= 1e-3


def test_edge_cases(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import events, fuzz, generator, native
    good = _sorted(oracle_lib, generator.generate(range(3))[0])
    ev = events.unpack_event(good[1])
    ev.y[5] = np.inf
    nonfinite = events.pack_event(ev)
    # module tables that do not tile [0, H): checked on the device
    raw = np.frombuffer(good[1], np.int32).copy()
    S = int(raw[0])
    gap = raw.copy()
    gap[2 + 2 * S + 7] -= 1                                # module 7 one hit short: starts stop lining up
    over = raw.copy()
    over[2 + 2 * S + S - 1] += 1                           # last module runs past H
    batch = [good[0], fuzz.empty_event(), nonfinite, b"\x05\x00\x00\x00", fuzz.empty_event(0), good[2],
             gap.tobytes(), over.tobytes()]
    got, status = gpu_ctx.search(batch, allow_invalid=True)
    assert status[2] & native.EVENT_INVALID and status[3] & native.EVENT_INVALID
    assert status[6] & native.EVENT_INVALID and status[7] & native.EVENT_INVALID
    assert len(got[1]) == 0 and len(got[2]) == 0 and len(got[3]) == 0 and len(got[4]) == 0
    assert len(got[6]) == 0 and len(got[7]) == 0
    pbuf, poffs, psizes = events.pack_events(batch)
    gpu_ctx.stage(pbuf, poffs, psizes)
    gpu_ctx.sort_staged()
    staged = gpu_ctx.fetch_staged(len(pbuf))
    for k in (6, 7):                                          # the device sort leaves them alone
        a, n = int(poffs[k]), int(psizes[k])
        assert bytes(staged[a:a + n]) == batch[k]
    want, _ = oracle_lib.search([good[0], good[2]], 4)
    assert index_lists(got[0]) == index_lists(want[0])
    assert index_lists(got[5]) == index_lists(want[1])
    with pytest.raises(native.VeloError):
        gpu_ctx.search(batch)                                  # strict call reports the bad events
    out, st = gpu_ctx.search([])
    assert out == [] and len(st) == 0
    # batch descriptions that are rejected before anything is copied
    for offs, sizes in (([2], [len(good[0])]),                       # offset not 4-byte aligned
                        ([8], [np.iinfo(np.uint64).max - 4])):        # offset + size wraps around
        with pytest.raises(native.VeloError) as err:
            gpu_ctx.stage(pbuf, np.array(offs, np.uint64), np.array(sizes, np.uint64))
        assert err.value.status == native.ERR_INVALID_ARGUMENT
    got, _ = gpu_ctx.search([good[0]])                                 # the context still works
    assert index_lists(got[0]) == index_lists(want[0])


def test_context_reuse_is_stable(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator
    small = _sorted(oracle_lib, generator.generate(range(800, 805))[0])
    big = _sorted(oracle_lib, generator.generate(range(810, 900))[0])
    a, _ = gpu_ctx.search(small)
    gpu_ctx.search(big)
    b, _ = gpu_ctx.search(small)
    assert [index_lists(x) for x in a] == [index_lists(x) for x in b]


def test_split_stage_run_fetch(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import events, generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(900, 930))[0])
    buf, offs, sizes = events.pack_events(blobs)
    gpu_ctx.stage(buf, offs, sizes)
    gpu_ctx.run(native.default_options(launch_mode=1))
    cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs))
    tracks, counts, first, status = gpu_ctx.fetch(len(blobs), cap)
    want, _ = oracle_lib.search(blobs, 4)
    for e in range(len(blobs)):
        assert index_lists(tracks[int(first[e]):int(first[e]) + int(counts[e])]) == index_lists(want[e])
    s = gpu_ctx.stats()
    assert s.launches == 1 and s.n_events == len(blobs) and s.total_tracks == counts.sum()
    assert gpu_ctx.time_runs(native.default_options(), warmup=1, iters=2, flush_l2=True) > 0


def test_device_sort_matches_reference_sort(gpu_ctx, oracle_lib, golden):
    """velo_sort_staged: the reference's preorder_by_x permutation, ties included."""
    from cl_forward_gb300 import fuzz, generator
    for name in ("velo", "fuzz", "edge"):
        raw = golden[name]["input"]
        _, _, sorted_blobs = gpu_ctx.search_unsorted(raw)
        assert sorted_blobs == golden[name]["sorted"], name
    raw = generator.generate(range(2000, 2030))[0] + [fuzz.fuzz_event(s, grid=2.0) for s in range(30)]
    got, status, sorted_blobs = gpu_ctx.search_unsorted(raw)
    assert sorted_blobs == [oracle_lib.sort_by_x(b) for b in raw]
    want, _ = oracle_lib.search(sorted_blobs, 4)
    for e in range(len(raw)):
        if not (status[e] & OVERFLOW_BITS):
            assert index_lists(got[e]) == index_lists(want[e])


def test_device_sort_of_sorted_crowded_modules(gpu_ctx, oracle_lib):
    """Sorting events a second time gives the reference's sort of the sorted
    bytes: the same bytes where a module's x values are distinct, and not
    where they tie (the reference's partition swaps equal neighbours on
    every pass).  Modules already in strictly increasing order take one pass:
    with 16,383-hit modules the reference's first-element pivots would walk
    ~1.3e8 steps in one thread each."""
    import time
    from cl_forward_gb300 import events, fuzz, generator
    distinct = []
    for s, m in ((1, 38), (2, 39), (3, 20)):
        ev = events.unpack_event(fuzz.crowded_event(s, 16383, module=m))
        rng = np.random.Generator(np.random.PCG64(s))          # every x of the event distinct
        x = np.unique(rng.uniform(-40, 40, 3 * ev.n_hits).astype(np.float32))
        ev.x[:] = rng.permutation(x)[:ev.n_hits]
        distinct.append(events.pack_event(ev))
    ties = [fuzz.crowded_event(4, 3000, module=30)] + [fuzz.fuzz_event(s, grid=2.0) for s in range(6)]
    raw = distinct + ties + generator.generate(range(2100, 2110))[0]
    once = [oracle_lib.sort_by_x(b) for b in raw]
    twice = [oracle_lib.sort_by_x(b) for b in once]
    assert twice[:3] == once[:3] and twice[3] != once[3]     # distinct x: fixed point; ties: not
    for batch, expect in ((raw, once), (once, twice), (once[:3], once[:3])):
        buf, offs, sizes = events.pack_events(batch)
        gpu_ctx.stage(buf, offs, sizes)
        gpu_ctx.synchronize()
        t0 = time.perf_counter()
        gpu_ctx.sort_staged()
        gpu_ctx.synchronize()
        dt = time.perf_counter() - t0
        staged = gpu_ctx.fetch_staged(len(buf))
        got = [bytes(staged[int(o):int(o) + int(n)]) for o, n in zip(offs, sizes)]
        assert got == expect
    assert dt < 0.1, f"re-sorting sorted 16,383-hit modules took {dt * 1e3:.1f} ms"


def test_track_fits_match_least_squares(gpu_ctx, oracle_lib):
    """velo_fit_tracks against a float64 least-squares fit (tolerance 1e-4 mm, 1e-6 in slope)."""
    from cl_forward_gb300 import events, generator
    blobs = [oracle_lib.sort_by_x(b) for b in generator.generate(range(3000, 3020))[0]]
    buf, offs, sizes = events.pack_events(blobs)
    gpu_ctx.stage(buf, offs, sizes)
    gpu_ctx.run()
    cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs))
    tracks, counts, first, _ = gpu_ctx.fetch(len(blobs), cap)
    fits = gpu_ctx.fit_tracks(cap)
    checked = 0
    for e, blob in enumerate(blobs):
        ev = events.unpack_event(blob)
        for i in range(int(counts[e])):
            t = tracks[int(first[e]) + i]
            h = t["hits"][:int(t["hitsNum"])]
            z = ev.z[h].astype(np.float64)
            A = np.stack([np.ones_like(z), z], 1)
            (x0, tx), *_ = np.linalg.lstsq(A, ev.x[h].astype(np.float64), rcond=None)
            (y0, ty), *_ = np.linalg.lstsq(A, ev.y[h].astype(np.float64), rcond=None)
            f = fits[int(first[e]) + i]
            assert abs(f["tx"] - tx) < 1e-6 + 1e-5 * abs(tx) and abs(f["ty"] - ty) < 1e-6 + 1e-5 * abs(ty)
            assert abs(f["x0"] - x0) < 1e-4 + 1e-5 * abs(x0) and abs(f["y0"] - y0) < 1e-4 + 1e-5 * abs(y0)
            r = np.concatenate([ev.x[h] - (x0 + tx * z), ev.y[h] - (y0 + ty * z)])
            chi2 = 3966.94 * float(r @ r) / (2 * len(h) - 4)
            assert abs(f["chi2_ndf"] - chi2) <= 1e-3 * max(chi2, 1e-3) + 1e-4
            checked += 1
    assert checked > 1000


@pytest.mark.parametrize("part,mode", [(128, 0), (100, 1)])
def test_pipelined_search_matches_one_launch(gpu_ctx, oracle_lib, part, mode):
    """Batches cut into overlapped parts on two streams: the same tracks per
    event, first[] rebased into one output array, statuses and the strict
    call's error for an invalid event kept."""
    from cl_forward_gb300 import events, fuzz, generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(5000, 5650))[0])
    blobs[333] = b"\x05\x00\x00\x00"                        # invalid, in a middle part
    blobs[400] = fuzz.empty_event()
    one, st1 = gpu_ctx.search(blobs, native.default_options(launch_mode=mode), allow_invalid=True)
    piped, st2 = gpu_ctx.search(blobs, native.default_options(launch_mode=mode, pipeline_events=part),
                                allow_invalid=True)
    assert np.array_equal(st1, st2) and st2[333] & native.EVENT_INVALID
    for e in range(len(blobs)):
        assert index_lists(piped[e]) == index_lists(one[e])
    s = gpu_ctx.stats()
    assert s.launches == -(-len(blobs) // part) and s.total_tracks == sum(len(t) for t in piped)
    with pytest.raises(native.VeloError):
        gpu_ctx.search(blobs, native.default_options(pipeline_events=part))
    with pytest.raises(native.VeloError):                   # the parent holds no staged batch afterwards
        gpu_ctx.fit_tracks(16)


@pytest.mark.parametrize("part", [0, 96])
def test_host_direct_io_matches_copies(gpu_ctx, oracle_lib, part):
    """Events read and tracks written in place in pinned host memory (alone
    and with pipelined parts) give the copied path's tracks; pageable buffers
    fall back to copies; a short track buffer is reported, not overrun."""
    from cl_forward_gb300 import events, fuzz, generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(6000, 6400))[0])
    blobs[50] = fuzz.empty_event()
    buf, offs, sizes = events.pack_events(blobs)
    n = len(blobs)
    cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs))
    pinned = gpu_ctx.host_alloc(len(buf))
    pinned[:] = buf
    ptracks = gpu_ctx.host_alloc(cap * 100).view(events.TRACK_DTYPE)
    want, _ = oracle_lib.search(blobs, 4)
    for src, dst in ((pinned, ptracks), (buf, np.zeros(cap, events.TRACK_DTYPE))):
        for mode in (0, 1):
            o = native.default_options(launch_mode=mode, host_direct=1, pipeline_events=part)
            counts = np.zeros(n, np.uint32)
            first = np.zeros(n, np.uint64)
            status = np.zeros(n, np.uint32)
            dst.view(np.uint8)[:] = 0
            gpu_ctx.search_packed_into(src, offs, sizes, o, dst, counts, first, status)
            assert not np.any(status & native.EVENT_INVALID)
            for e in range(n):
                assert index_lists(dst[int(first[e]):int(first[e]) + int(counts[e])]) == index_lists(want[e])
            assert int((first + counts).max()) == int(counts.sum())          # one contiguous range
    total = sum(len(t) for t in want)
    with pytest.raises(native.VeloError):
        o = native.default_options(host_direct=1, pipeline_events=part)
        gpu_ctx.search_packed_into(pinned, offs, sizes, o, ptracks[:total - 1], np.zeros(n, np.uint32),
                                   np.zeros(n, np.uint64), np.zeros(n, np.uint32))
    gpu_ctx.host_free(pinned)
    gpu_ctx.host_free(ptracks.view(np.uint8))


def test_device_budget_splits_large_batches(gpu_ctx, oracle_lib):
    """A batch needing more device memory than the call's budget is cut into
    pipelined parts: same tracks and statuses, one contiguous output."""
    from cl_forward_gb300 import generator, native
    blobs = _sorted(oracle_lib, generator.generate(range(7000, 7300))[0])
    whole, st1 = gpu_ctx.search(blobs, native.default_options())
    for direct in (0, 1):
        parts, st2 = gpu_ctx.search(blobs, native.default_options(device_budget_mb=8, host_direct=direct))
        assert np.array_equal(st1, st2)
        assert gpu_ctx.stats().launches > 2                  # it was split
        for e in range(len(blobs)):
            assert index_lists(parts[e]) == index_lists(whole[e])


def test_many_module_events_take_the_full_build(gpu_ctx, oracle_lib):
    """Events with 64 or more modules run on the full shared-state build (the
    compact one holds 63), alone and mixed with ordinary events, for every
    register build and launch style."""
    from cl_forward_gb300 import fuzz, generator
    wide = [oracle_lib.sort_by_x(fuzz.fuzz_event(9000 + s, n_modules=n, max_per_module=10, grid=0.5, lines=8))
            for s, n in enumerate((64, 80, 120, 255, 100, 70))]
    mixed = wide + _sorted(oracle_lib, generator.generate(range(9100, 9110))[0])
    for blobs in (wide, mixed):
        for regs, threads in ((18, 64), (4, 128), (5, 256)):
            for mode in (0, 1):
                _assert_same(gpu_ctx, oracle_lib, blobs, register_ctas=regs, threads_per_event=threads,
                             launch_mode=mode)


def test_maximum_module_occupancy(gpu_ctx, oracle_lib):
    """Modules holding the most hits a module may hold (16,383): on modules 38
    and 39 (50 mm from the h0 modules above them) an h0's h1 window spans
    ~14,000 hits, near the top of the seeding key's 14-bit element field.
    Every launch style gives the oracle's tracks; a module of one hit more
    makes its event invalid and leaves the rest of the batch alone."""
    from cl_forward_gb300 import fuzz, native
    full = [oracle_lib.sort_by_x(fuzz.crowded_event(s, 16383, module=m)) for s, m in ((1, 38), (2, 39), (3, 20))]
    for regs, threads in ((18, 64), (5, 256)):
        for mode in (0, 1):
            _, checked = _assert_same(gpu_ctx, oracle_lib, full, register_ctas=regs, threads_per_event=threads,
                                      launch_mode=mode)
            assert checked == 3
    over = fuzz.crowded_event(1, 16384, module=38)
    got, status = gpu_ctx.search([full[0], over, full[2]], allow_invalid=True)
    want, _ = oracle_lib.search([full[0], full[2]], 4)
    assert status[1] & native.EVENT_INVALID and len(got[1]) == 0
    assert index_lists(got[0]) == index_lists(want[0]) and index_lists(got[2]) == index_lists(want[1])


def test_contexts_in_concurrent_threads(gpu_ctx, oracle_lib):
    """One context per host thread: four threads searching different batches
    at the same time (the library's calls release the interpreter) get the
    tracks a single thread gets."""
    import threading
    from cl_forward_gb300 import generator, native
    batches = [_sorted(oracle_lib, generator.generate(range(9500 + 100 * k, 9560 + 100 * k))[0]) for k in range(4)]
    want = [gpu_ctx.search(b)[0] for b in batches]
    got = [None] * 4
    errors = []

    def work(k):
        try:
            with native.Context(0) as ctx:
                for _ in range(3):
                    got[k] = ctx.search(batches[k], native.default_options(host_direct=k % 2))[0]
        except Exception as exc:   # reported below, on the main thread
            errors.append(exc)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k in range(4):
        assert [index_lists(t) for t in got[k]] == [index_lists(t) for t in want[k]]
