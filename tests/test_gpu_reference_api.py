"""The reference-signature entry points (Python mirror and C++ driver) on the GPU."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import index_lists

pytestmark = pytest.mark.gpu


def test_python_mirror_independent_execute(native_lib, oracle_lib):
    from cl_forward_gb300 import generator, search
    raw = generator.generate(range(40, 60))[0]
    inp = [bytearray(b) for b in raw]
    out = []
    assert search.independent_execute(inp, out) == 0
    assert len(out) == len(raw)
    sorted_blobs = [oracle_lib.sort_by_x(b) for b in raw]
    assert [bytes(b) for b in inp] == sorted_blobs            # sorted in place, like the reference
    want, _ = oracle_lib.search(sorted_blobs, 4)
    for e in range(len(raw)):
        assert len(out[e]) % 100 == 0
        assert index_lists(search.tracks_of(out[e])) == index_lists(want[e])
    out2 = []
    search.gpuPixelSearchByTriplet(sorted_blobs, out2)
    assert out2 == out or all(index_lists(search.tracks_of(a)) == index_lists(search.tracks_of(b))
                              for a, b in zip(out, out2))


def test_invoke_parallel_search_window(native_lib, oracle_lib):
    from cl_forward_gb300 import generator, search
    blobs = [oracle_lib.sort_by_x(b) for b in generator.generate(range(60, 70))[0]]
    out = [b"untouched"] * len(blobs)
    search.invokeParallelSearch(3, 4, blobs, out)
    assert out[:3] == [b"untouched"] * 3 and out[7:] == [b"untouched"] * 3
    want, _ = oracle_lib.search(blobs[3:7], 4)
    for i in range(4):
        assert index_lists(search.tracks_of(out[3 + i])) == index_lists(want[i])


def test_cpp_driver_dump(native_lib, oracle_lib, tmp_path):
    from cl_forward_gb300 import build, events, generator
    raw = generator.generate(range(70, 73))[0]
    data = tmp_path / "data"
    dump = tmp_path / "dump"
    data.mkdir()
    dump.mkdir()
    for i, b in enumerate(raw):
        events.write_dat(str(data / f"{i}.dat"), b)
    r = subprocess.run([build.DRIVER, str(data), "3", "--dump", str(dump)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "3 files read" in r.stdout
    want, _ = oracle_lib.search([oracle_lib.sort_by_x(b) for b in raw], 4)
    for i in range(3):
        text = (dump / f"{i}.out").read_text()
        tracks = re.findall(r"Track #(\d+), length (\d+)\n(.*?)\n\n", text, re.S)
        assert len(tracks) == len(want[i])
        ids = sorted(tuple(sorted(int(m) for m in re.findall(r"^\s+(\d+) \(", body, re.M)))
                     for _, _, body in tracks)
        ev = events.unpack_event(oracle_lib.sort_by_x(raw[i]))
        ref_ids = sorted(tuple(sorted(int(ev.hit_id[h]) for h in t)) for t in index_lists(want[i]))
        assert ids == ref_ids
        from cl_forward_gb300 import compare                 # the dump reader sees the same tracks
        assert sorted(tuple(sorted(t)) for t in compare.read_dump(str(dump / f"{i}.out"))) == ref_ids


def test_cpp_driver_sorts_many_events_in_parallel(native_lib, oracle_lib, tmp_path):
    """independent_execute through the C++ driver on 150 events: the events
    are sorted on the GPU (velo_sort_staged) with the reference's
    permutation, so the dumped tracks match the oracle's on the sorted events."""
    from cl_forward_gb300 import build, events, generator
    raw = generator.generate(range(300, 450))[0]
    data = tmp_path / "data"
    dump = tmp_path / "dump"
    data.mkdir()
    dump.mkdir()
    for i, b in enumerate(raw):
        events.write_dat(str(data / f"{i:03d}.dat"), b)
    r = subprocess.run([build.DRIVER, str(data), str(len(raw)), "--dump", str(dump)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    want, _ = oracle_lib.search([oracle_lib.sort_by_x(b) for b in raw], 4)
    names = sorted(os.listdir(str(data)))
    for i, name in enumerate(names):
        e = int(name.split(".")[0])
        text = (dump / f"{i}.out").read_text()
        tracks = re.findall(r"Track #(\d+), length (\d+)\n(.*?)\n\n", text, re.S)
        ids = sorted(tuple(sorted(int(m) for m in re.findall(r"^\s+(\d+) \(", body, re.M)))
                     for _, _, body in tracks)
        ev = events.unpack_event(oracle_lib.sort_by_x(raw[e]))
        assert ids == sorted(tuple(sorted(int(ev.hit_id[h]) for h in t)) for t in index_lists(want[e]))


def test_reference_entry_points_on_vectors(native_lib, oracle_lib):
    """The reference-signature entry points on std::vector input, through the
    timing harness: independent_execute leaves the caller's buffers sorted
    byte for byte as the reference's preorder_by_x does (Tools.cpp:46-66);
    its output vectors and gpuPixelSearchByTriplet's on the sorted events
    hold the oracle's tracks, event by event.  20,000 events: two chunks of
    at most 16,000 (GpuPixelSearchByTriplet.cpp:53)."""
    from cl_forward_gb300 import generator, native, validation
    raw = generator.generate_parallel(range(20000, 40000))[0]
    ms, tracks_ie, dig_ie, after = native.reference_api_times(raw, "independent_execute", 0, 1, want_sorted=True)
    want_sorted = [oracle_lib.sort_by_x(b) for b in raw]
    assert after == want_sorted
    ms2, tracks_gp, dig_gp, untouched = native.reference_api_times(want_sorted, "gpuPixelSearchByTriplet", 0, 1,
                                                                   want_sorted=True)
    assert untouched == want_sorted                    # the framework entry does not sort
    assert tracks_ie == tracks_gp and np.array_equal(dig_ie, dig_gp)
    want, wst = oracle_lib.search(want_sorted, 4)
    words = np.concatenate([w.view(np.uint32).reshape(-1, 25) for w in want])
    ohash = validation.event_hashes(words, np.array([len(w) for w in want]))
    compared = np.flatnonzero((wst & oracle_lib.PARITY_EXCLUDING) == 0)
    assert len(compared) > 19900
    assert np.array_equal(dig_gp[compared], ohash[compared])
    assert ms[0] > 0 and ms2[0] > 0


@pytest.mark.parametrize("direct", [0, 1])
def test_sort_search_sorts_in_place(gpu_ctx, oracle_lib, direct):
    """velo_sort_search: the caller's buffers end up sorted byte for byte as
    the reference's preorder_by_x leaves them (ties included: the fuzz events
    put several hits at one x), and the tracks are the oracle's.  host_direct
    1 lets a device with coherent access to pageable memory sort the buffers
    where they lie; 0 sorts a pinned copy and copies the bytes back."""
    from cl_forward_gb300 import fuzz, generator, native
    raw = generator.generate(range(60, 140))[0] + [fuzz.fuzz_event(s, grid=2.0) for s in range(40)]
    raw += [fuzz.crowded_event(4, 3000, module=30), fuzz.empty_event()]
    bufs = [bytearray(b) for b in raw]
    got, status = gpu_ctx.sort_search(bufs, native.default_options(host_direct=direct))
    want_sorted = [oracle_lib.sort_by_x(b) for b in raw]
    assert [bytes(b) for b in bufs] == want_sorted
    want, wst = oracle_lib.search(want_sorted, 4)
    assert np.array_equal(status & 0x7, wst & 0x7)
    for e in range(len(raw)):
        if not (wst[e] & oracle_lib.PARITY_EXCLUDING):
            assert index_lists(got[e]) == index_lists(want[e]), e
    # a second call sorts the sorted bytes again, as the reference would: a
    # fixed point where x values are distinct, another permutation of equal x
    again_sorted = [oracle_lib.sort_by_x(b) for b in want_sorted]
    again, _ = gpu_ctx.sort_search(bufs, native.default_options(host_direct=direct))
    assert [bytes(b) for b in bufs] == again_sorted
    want2, wst2 = oracle_lib.search(again_sorted, 4)
    for e in range(len(raw)):
        if not (wst2[e] & oracle_lib.PARITY_EXCLUDING):
            assert index_lists(again[e]) == index_lists(want2[e]), e


def test_sort_search_rejects_misaligned_buffers(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator, native
    blob = generator.generate([5])[0][0]
    raw = bytearray(len(blob) + 1)
    view = np.frombuffer(raw, np.uint8)[1:]
    view[:] = np.frombuffer(blob, np.uint8)
    with pytest.raises(native.VeloError) as err:
        gpu_ctx.sort_search([view], native.default_options(host_direct=1))
    assert err.value.status == native.ERR_INVALID_ARGUMENT
    assert bytes(view) == blob                          # untouched


@pytest.mark.parametrize("sort", [0, 1])
def test_streamed_results(gpu_ctx, oracle_lib, sort):
    """velo_search_begin / velo_search_end: every event's record becomes ready
    while or after the device searches, its tracks are in place once it is,
    and records, tracks and the end call's outputs equal the synchronous
    search's (with sort, after the in-place sort of the caller's buffers)."""
    import time
    from cl_forward_gb300 import fuzz, generator, native
    raw = generator.generate(range(200, 500))[0] + [fuzz.fuzz_event(s, grid=2.0) for s in range(20)]
    raw += [fuzz.empty_event()]
    want_sorted = [oracle_lib.sort_by_x(b) for b in raw]
    bufs = [bytearray(b) for b in (raw if sort else want_sorted)]
    results, tracks, keep = gpu_ctx.search_begin(bufs, sort=bool(sort))
    t0 = time.perf_counter()
    while not results["ready"].all():
        assert time.perf_counter() - t0 < 60, "records not ready"
        time.sleep(0.0005)
    got = [tracks[int(r["first"]):int(r["first"]) + int(r["count"])].copy() for r in results]
    counts, first, status = gpu_ctx.search_end(len(bufs))
    assert np.array_equal(counts, results["count"]) and np.array_equal(first, results["first"])
    assert np.array_equal(status, results["status"])
    assert [bytes(b) for b in bufs] == want_sorted
    want, wst = oracle_lib.search(want_sorted, 4)
    assert np.array_equal(status & 0x7, wst & 0x7)
    for e in range(len(raw)):
        if not (wst[e] & oracle_lib.PARITY_EXCLUDING):
            assert index_lists(got[e]) == index_lists(want[e]), e
    del keep


def test_streamed_search_call_order(gpu_ctx, oracle_lib):
    from cl_forward_gb300 import generator, native
    bufs = [bytearray(oracle_lib.sort_by_x(b)) for b in generator.generate(range(600, 610))[0]]
    with pytest.raises(native.VeloError) as err:
        gpu_ctx.search_end(len(bufs))                       # nothing in flight
    assert err.value.status == native.ERR_NOT_STAGED
    results, tracks, keep = gpu_ctx.search_begin(bufs)
    with pytest.raises(native.VeloError) as err:
        gpu_ctx.search_begin(bufs)                          # one streamed search at a time
    assert err.value.status == native.ERR_INVALID_ARGUMENT
    for call in (lambda: gpu_ctx.search(bufs), lambda: gpu_ctx.run(), lambda: gpu_ctx.fetch_counts(len(bufs)),
                 lambda: gpu_ctx.sort_search([bytearray(b) for b in bufs])):
        with pytest.raises(native.VeloError) as err:        # the in-flight search owns the context
            call()
        assert err.value.status == native.ERR_INVALID_ARGUMENT
    counts, _, _ = gpu_ctx.search_end(len(bufs))
    assert results["ready"].all() and np.array_equal(counts, results["count"])
    got, _ = gpu_ctx.search(bufs)                            # the context works on
    assert [len(g) for g in got] == counts.tolist()
    del keep
