"""The C-ABI library builds, loads and exports every declared symbol.

Host-only entry points (validation, the reference x-sort, capacity) are
exercised here; nothing in this file needs a GPU.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(velo_[a-z_]+)\s*\(", src)))


def _exported(lib_path, demangle=False):
    out = subprocess.run(["nm", "-D", "--defined-only"] + (["-C"] if demangle else []) + [lib_path],
                         capture_output=True, text=True, check=True).stdout
    return out


def test_every_c_abi_symbol_is_exported(native_lib):
    from cl_forward_gb300 import native
    names = _declared("velo_search.h")
    assert len(names) >= 15
    assert sorted(native.EXPORTED) == names
    syms = set(l.split()[-1] for l in _exported(native.lib_path()).splitlines())
    missing = [n for n in names if n not in syms]
    assert not missing
    for n in names:
        assert getattr(native_lib, n) is not None


def test_reference_cpp_entry_points_are_exported(native_lib):
    from cl_forward_gb300 import native
    out = _exported(native.lib_path(), demangle=True)
    for sym in ("invokeParallelSearch(int, int,", "gpuPixelSearchByTriplet(std::vector",
                "gpuPixelSearchByTripletInvocation(", "independent_execute(", "independent_post_execute(",
                "preorder_by_x("):
        assert sym in out, sym


def test_reference_api_timing_harness_builds(native_lib):
    """bench.py's harness for the reference-signature entry points loads (it
    links the library) and exports its one timing call."""
    import ctypes
    from cl_forward_gb300 import native
    assert os.path.exists(native.API_BENCH_PATH)
    assert "velo_bench_reference_api" in _exported(native.API_BENCH_PATH)
    lib = ctypes.CDLL(native.API_BENCH_PATH)
    lib.velo_bench_reference_api.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 4
    assert lib.velo_bench_reference_api(None, None, None, -1, 0, 0, 1, None, None, None, None) == -1
    assert lib.velo_bench_reference_api(None, None, None, 0, 2, 0, 1, None, None, None, None) == -1


def test_seed_lanes_field_keeps_the_options_layout():
    """seed_lanes took one of the reserved words: the structure is 64 bytes."""
    import ctypes
    from cl_forward_gb300 import native
    assert ctypes.sizeof(native.Options) == 64
    assert native.Options.seed_lanes.offset == 48


def test_no_forbidden_cuda_calls_in_sources():
    bad = re.compile(r"cu(da)?Memcpy(3D)?BatchAsync")
    for d in ("cl_forward_gb300/csrc", "include"):
        for f in os.listdir(os.path.join(ROOT, d)):
            assert not bad.search(open(os.path.join(ROOT, d, f), errors="ignore").read()), f


def test_validate_event(native_lib):
    from cl_forward_gb300 import events, generator, native
    blob = generator.generate([1])[0][0]
    assert native.validate_event(blob) == native.OK
    assert native.validate_event(blob[:-4]) == native.ERR_INVALID_EVENT     # truncated
    assert native.validate_event(b"") == native.ERR_INVALID_EVENT
    ev = events.unpack_event(blob)
    ev.hit_start[3] += 1                                                   # non-contiguous modules
    assert native.validate_event(events.pack_event(ev)) == native.ERR_INVALID_EVENT
    ev = events.unpack_event(blob)
    ev.x[10] = np.nan
    assert native.validate_event(events.pack_event(ev)) == native.ERR_INVALID_EVENT
    ev = events.unpack_event(blob)
    bad = bytearray(events.pack_event(ev))
    bad[0:4] = (300).to_bytes(4, "little")                                 # too many modules
    assert native.validate_event(bytes(bad)) == native.ERR_INVALID_EVENT
    from cl_forward_gb300 import fuzz                                      # module occupancy limit
    assert native.validate_event(fuzz.crowded_event(1, 16383)) == native.OK
    assert native.validate_event(fuzz.crowded_event(1, 16384)) == native.ERR_INVALID_EVENT


def test_native_sort_matches_oracle_sort(native_lib, oracle_lib, golden):
    for name in ("velo", "fuzz", "edge"):
        for raw, ref_sorted in zip(golden[name]["input"], golden[name]["sorted"]):
            assert oracle_lib.sort_by_x(raw) == ref_sorted
            if len(raw) >= 8:
                from cl_forward_gb300 import native
                assert native.sort_by_x(raw) == ref_sorted


def test_python_mirror_sort_in_place(native_lib, golden):
    from cl_forward_gb300 import search
    bufs = [bytearray(b) for b in golden["velo"]["input"]]
    search.preorder_by_x(bufs)
    assert [bytes(b) for b in bufs] == golden["velo"]["sorted"]
    with pytest.raises(TypeError):
        search.preorder_by_x([bytes(golden["velo"]["input"][0])])


def test_track_capacity(native_lib):
    import ctypes
    from cl_forward_gb300 import generator
    blobs = generator.generate(range(3))[0] + [b""]
    arrs = [np.frombuffer(b, np.uint8) for b in blobs]
    ptrs = (ctypes.c_void_p * len(blobs))(*[a.ctypes.data if len(a) else 0 for a in arrs])
    sizes = np.array([len(b) for b in blobs], np.uint64)
    cap = native_lib.velo_track_capacity(ptrs, sizes.ctypes.data, len(blobs))
    expect = sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) for b in blobs[:3]) + 1
    assert cap == expect


def test_context_without_gpu_fails_loudly(native_lib):
    from cl_forward_gb300 import native
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(native.VeloError):
        native.Context(0)


def test_default_options(native_lib):
    from cl_forward_gb300 import native
    o = native.default_options()
    assert o.y_lanes == 4 and o.threads_per_event == 64 and o.narrow_windows == 1
    assert o.launch_mode == native.LAUNCH_PERSISTENT and o.smem_hits == 50 and o.register_ctas == 0
    assert o.learned == 0 and o.pipeline_events == 0 and o.host_direct == 0 and o.use_graph == 0
    o = native.default_options(y_lanes=2, launch_mode=native.LAUNCH_PER_EVENT)
    assert o.y_lanes == 2 and o.launch_mode == 0


def test_python_mirror_refuses_immutable_input():
    """The reference sorts its input in place: the Python mirror's
    independent_execute and preorder_by_x refuse `bytes` (immutable) before
    any device work."""
    from cl_forward_gb300 import generator, search
    blob = generator.generate([3])[0][0]
    with pytest.raises(TypeError):
        search.independent_execute([blob], [])
    with pytest.raises(TypeError):
        search.preorder_by_x([blob])
    buf = bytearray(blob)
    search.preorder_by_x([buf])                      # host sort, no GPU needed
    from oracle import oracle
    oracle.build()
    assert bytes(buf) == oracle.sort_by_x(blob)
