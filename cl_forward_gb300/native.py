"""ctypes binding of ``libclforward_gb300.so`` (the C ABI in include/velo_search.h).

The library is the only compute path: if it has not been built, or no CUDA
device is present, the calls that need it raise; there is no CPU fallback.
Host-only helpers (validation, the reference x-sort) work without a GPU.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from .events import TRACK_DTYPE

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libclforward_gb300.so")

# velo_status
OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_INVALID_EVENT = -2
ERR_CAPACITY = -3
ERR_CUDA = -4
ERR_TIMEOUT = -5            # reserved (no entry point returns it)
ERR_NO_DEVICE = -6
ERR_OUT_OF_MEMORY = -7
ERR_NOT_STAGED = -8

# per-event status bits
EVENT_RING_OVERFLOW = 0x1
EVENT_TRACK_OVERFLOW = 0x2
EVENT_MAX_TRACKS = 0x4
EVENT_INVALID = 0x8
EVENT_DEGENERATE = 0x10

LAUNCH_PER_EVENT = 0
LAUNCH_PERSISTENT = 1

# every symbol include/velo_search.h declares
EXPORTED = [
    "velo_default_options", "velo_status_string", "velo_create", "velo_destroy", "velo_last_error",
    "velo_validate_event", "velo_sort_by_x", "velo_track_capacity", "velo_search",
    "velo_search_packed", "velo_stage", "velo_run", "velo_fetch", "velo_synchronize",
    "velo_get_stats", "velo_time_runs", "velo_host_alloc", "velo_host_free", "velo_device_sm_count",
    "velo_search_device_static", "velo_autotune", "velo_set_mlp", "velo_dump_doublets",
    "velo_mlp_train", "velo_mlp_grad", "velo_mlp_forward", "velo_sort_staged", "velo_fetch_staged",
    "velo_fit_tracks", "velo_sort_search", "velo_search_begin", "velo_search_end",
]

# velo_event_result (32 bytes)
RESULT_DTYPE = np.dtype([("first", "<u8"), ("count", "<u4"), ("status", "<u4"), ("ready", "<u4"),
                         ("reserved", "<u4", 3)])

FIT_DTYPE = np.dtype([("x0", "<f4"), ("tx", "<f4"), ("y0", "<f4"), ("ty", "<f4"), ("chi2_ndf", "<f4")])

MLP_INPUTS = 10
MLP_HIDDEN = 32
MLP_PARAMS = 1474
EVENT_LEARNED_FALLBACK = 0x20

# limits of velo_search_device_static (include/velo_search.h)
STATIC_MAX_EVENTS = 4096
STATIC_MAX_HIT_ROWS = 131072


class Options(ctypes.Structure):
    _fields_ = [("y_lanes", ctypes.c_int32), ("threads_per_event", ctypes.c_int32),
                ("launch_mode", ctypes.c_int32), ("smem_hits", ctypes.c_int32),
                ("narrow_windows", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("use_graph", ctypes.c_int32), ("register_ctas", ctypes.c_int32),
                ("learned", ctypes.c_int32), ("pipeline_events", ctypes.c_int32),
                ("host_direct", ctypes.c_int32), ("device_budget_mb", ctypes.c_int32),
                ("seed_lanes", ctypes.c_int32), ("learned_min_window", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 2)]


class Stats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_float), ("launches", ctypes.c_uint32),
                ("n_events", ctypes.c_uint32), ("total_hits", ctypes.c_uint64),
                ("total_tracks", ctypes.c_uint64), ("input_bytes", ctypes.c_uint64),
                ("output_bytes", ctypes.c_uint64), ("smem_bytes_per_cta", ctypes.c_int32),
                ("grid", ctypes.c_int32), ("block", ctypes.c_int32),
                ("events_in_global", ctypes.c_int32), ("host_stage_ms", ctypes.c_float),
                ("host_launch_ms", ctypes.c_float), ("host_fetch_ms", ctypes.c_float)]


class VeloError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None


def lib_path() -> str:
    return LIB_PATH


def load() -> ctypes.CDLL:
    """Load the native library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"native library missing: {LIB_PATH}; run cl_forward_gb300.build.build()")
    l = ctypes.CDLL(LIB_PATH)
    vp, i32, u64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64
    l.velo_default_options.argtypes = [ctypes.POINTER(Options)]
    l.velo_default_options.restype = None
    l.velo_status_string.argtypes = [ctypes.c_int]
    l.velo_status_string.restype = ctypes.c_char_p
    l.velo_create.argtypes = [ctypes.POINTER(vp), i32]
    l.velo_destroy.argtypes = [vp]
    l.velo_destroy.restype = None
    l.velo_last_error.argtypes = [vp]
    l.velo_last_error.restype = ctypes.c_char_p
    l.velo_validate_event.argtypes = [vp, u64]
    l.velo_sort_by_x.argtypes = [vp, u64]
    l.velo_track_capacity.argtypes = [vp, vp, i32]
    l.velo_track_capacity.restype = u64
    l.velo_search.argtypes = [vp, vp, vp, i32, ctypes.POINTER(Options), vp, u64, vp, vp, vp]
    l.velo_search_packed.argtypes = [vp, vp, vp, vp, i32, ctypes.POINTER(Options), vp, u64, vp, vp, vp]
    l.velo_stage.argtypes = [vp, vp, vp, vp, i32]
    l.velo_run.argtypes = [vp, ctypes.POINTER(Options)]
    l.velo_fetch.argtypes = [vp, vp, u64, vp, vp, vp]
    l.velo_synchronize.argtypes = [vp]
    l.velo_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    l.velo_time_runs.argtypes = [vp, ctypes.POINTER(Options), i32, i32, i32, ctypes.POINTER(ctypes.c_float)]
    l.velo_host_alloc.argtypes = [vp, u64, ctypes.POINTER(vp)]
    l.velo_host_free.argtypes = [vp, vp]
    l.velo_device_sm_count.argtypes = [vp]
    l.velo_device_sm_count.restype = i32
    l.velo_search_device_static.argtypes = [vp, vp, vp, i32, u64, ctypes.c_uint32, i32, vp, u64, vp, vp, vp, vp]
    l.velo_autotune.argtypes = [vp, ctypes.POINTER(Options), i32, ctypes.POINTER(Options),
                                ctypes.POINTER(ctypes.c_float)]
    f32 = ctypes.c_float
    l.velo_set_mlp.argtypes = [vp, vp, f32, f32, f32, ctypes.c_uint32]
    l.velo_dump_doublets.argtypes = [vp, ctypes.POINTER(Options), ctypes.c_uint32, vp, vp, u64,
                                     ctypes.POINTER(u64)]
    l.velo_mlp_train.argtypes = [vp, vp, vp, ctypes.c_int64, i32, i32, f32, u64, vp, vp]
    l.velo_mlp_grad.argtypes = [vp, vp, vp, vp, ctypes.c_int64, vp, ctypes.POINTER(f32)]
    l.velo_mlp_forward.argtypes = [vp, vp, ctypes.c_int64, vp]
    l.velo_sort_staged.argtypes = [vp]
    l.velo_fetch_staged.argtypes = [vp, vp, u64]
    l.velo_fit_tracks.argtypes = [vp, vp, u64]
    l.velo_sort_search.argtypes = [vp, vp, vp, i32, ctypes.POINTER(Options), vp, u64, vp, vp, vp]
    l.velo_search_begin.argtypes = [vp, vp, vp, i32, ctypes.POINTER(Options), i32, vp, u64, vp]
    l.velo_search_end.argtypes = [vp, vp, vp, vp]
    _lib = l
    return l


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def default_options(**kw) -> Options:
    o = Options()
    load().velo_default_options(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, int(v))
    return o


def validate_event(blob: bytes) -> int:
    buf = np.frombuffer(blob, np.uint8)
    return int(load().velo_validate_event(_p(buf) if len(buf) else None, len(blob)))


def sort_by_x(blob: bytes) -> bytes:
    """The reference's per-module x-sort (Tools.cpp:46-66) of one event blob."""
    buf = np.frombuffer(bytearray(blob), np.uint8).copy()
    st = load().velo_sort_by_x(_p(buf), len(blob))
    if st != OK:
        raise VeloError(st, "velo_sort_by_x")
    return buf.tobytes()


class Context:
    """One CUDA stream and its device buffers (``velo_ctx``)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        self._h = ctypes.c_void_p()
        st = self._lib.velo_create(ctypes.byref(self._h), device)
        if st != OK:
            raise VeloError(st, f"velo_create: {self._lib.velo_status_string(st).decode()}")

    def close(self):
        if self._h:
            self._lib.velo_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int, what: str):
        if st != OK:
            detail = self._lib.velo_last_error(self._h).decode(errors="replace")
            raise VeloError(st, f"{what}: {self._lib.velo_status_string(st).decode()}: {detail}")

    @property
    def sm_count(self) -> int:
        return int(self._lib.velo_device_sm_count(self._h))

    # -- one-call host path ------------------------------------------------
    def search(self, blobs: Sequence[bytes], options: Optional[Options] = None, allow_invalid: bool = False):
        """Search x-sorted events.  Returns (list of per-event Track arrays, status uint32[n])."""
        n = len(blobs)
        arrs = [np.frombuffer(b, np.uint8) for b in blobs]
        ptrs = (ctypes.c_void_p * max(n, 1))(*[a.ctypes.data if len(a) else 0 for a in arrs])
        sizes = np.array([len(b) for b in blobs], np.uint64)
        cap = int(self._lib.velo_track_capacity(ptrs, _p(sizes), n))
        tracks = np.zeros(max(cap, 1), TRACK_DTYPE)
        counts = np.zeros(max(n, 1), np.uint32)
        first = np.zeros(max(n, 1), np.uint64)
        status = np.zeros(max(n, 1), np.uint32)
        opts = options or default_options()
        st = self._lib.velo_search(self._h, ptrs, _p(sizes), n, ctypes.byref(opts), _p(tracks), cap,
                                   _p(counts), _p(first), _p(status))
        if not (allow_invalid and st == ERR_INVALID_EVENT):
            self._check(st, "velo_search")
        out = [tracks[int(first[e]):int(first[e]) + int(counts[e])].copy() for e in range(n)]
        return out, status[:n].copy()

    def sort_search(self, blobs: Sequence[bytearray], options: Optional[Options] = None,
                    allow_invalid: bool = False):
        """velo_sort_search: sorts the events' modules by x in place (the
        caller's writable buffers, e.g. bytearrays) and searches them.
        Returns (list of per-event Track arrays, status uint32[n])."""
        n = len(blobs)
        arrs = [np.frombuffer(b, np.uint8) for b in blobs]
        for a in arrs:
            if len(a) and not a.flags.writeable:
                raise ValueError("sort_search sorts in place: pass writable buffers")
        ptrs = (ctypes.c_void_p * max(n, 1))(*[a.ctypes.data if len(a) else 0 for a in arrs])
        sizes = np.array([len(b) for b in blobs], np.uint64)
        cap = int(self._lib.velo_track_capacity(ptrs, _p(sizes), n))
        tracks = np.zeros(max(cap, 1), TRACK_DTYPE)
        counts = np.zeros(max(n, 1), np.uint32)
        first = np.zeros(max(n, 1), np.uint64)
        status = np.zeros(max(n, 1), np.uint32)
        opts = options or default_options()
        st = self._lib.velo_sort_search(self._h, ptrs, _p(sizes), n, ctypes.byref(opts), _p(tracks), cap,
                                        _p(counts), _p(first), _p(status))
        if not (allow_invalid and st == ERR_INVALID_EVENT):
            self._check(st, "velo_sort_search")
        out = [tracks[int(first[e]):int(first[e]) + int(counts[e])].copy() for e in range(n)]
        return out, status[:n].copy()

    def search_begin(self, blobs: Sequence[bytearray], sort: bool = False, options: Optional[Options] = None):
        """velo_search_begin: starts a search whose per-event results the
        device publishes as events finish.  Returns (results, tracks, keep):
        the RESULT_DTYPE records and the track buffer the device fills, and
        the objects to keep alive until :meth:`search_end`."""
        n = len(blobs)
        arrs = [np.frombuffer(b, np.uint8) for b in blobs]
        ptrs = (ctypes.c_void_p * max(n, 1))(*[a.ctypes.data if len(a) else 0 for a in arrs])
        sizes = np.array([len(b) for b in blobs], np.uint64)
        cap = int(self._lib.velo_track_capacity(ptrs, _p(sizes), n))
        tracks = np.zeros(max(cap, 1), TRACK_DTYPE)
        results = np.zeros(max(n, 1), RESULT_DTYPE)
        opts = options or default_options(host_direct=1)
        st = self._lib.velo_search_begin(self._h, ptrs, _p(sizes), n, ctypes.byref(opts), int(sort), _p(tracks),
                                         cap, _p(results))
        self._check(st, "velo_search_begin")
        return results[:n], tracks, (arrs, ptrs, sizes, opts)

    def search_end(self, n_events: int):
        counts = np.zeros(max(n_events, 1), np.uint32)
        first = np.zeros(max(n_events, 1), np.uint64)
        status = np.zeros(max(n_events, 1), np.uint32)
        self._check(self._lib.velo_search_end(self._h, _p(counts), _p(first), _p(status)), "velo_search_end")
        return counts[:n_events], first[:n_events], status[:n_events]

    # -- split path ----------------------------------------------------------
    def stage(self, buf: np.ndarray, offsets: np.ndarray, sizes: np.ndarray):
        self._staged = (buf, offsets, sizes)   # keep host memory alive until the copy is done
        self._check(self._lib.velo_stage(self._h, buf.ctypes.data, _p(offsets), _p(sizes), len(offsets)),
                    "velo_stage")

    def run(self, options: Optional[Options] = None):
        opts = options or default_options()
        self._check(self._lib.velo_run(self._h, ctypes.byref(opts)), "velo_run")

    def fetch(self, n_events: int, capacity: int):
        tracks = np.zeros(max(capacity, 1), TRACK_DTYPE)
        counts = np.zeros(max(n_events, 1), np.uint32)
        first = np.zeros(max(n_events, 1), np.uint64)
        status = np.zeros(max(n_events, 1), np.uint32)
        self._check(self._lib.velo_fetch(self._h, _p(tracks), capacity, _p(counts), _p(first), _p(status)),
                    "velo_fetch")
        return tracks, counts[:n_events], first[:n_events], status[:n_events]

    def fetch_counts(self, n_events: int):
        """Per-event counts, first rows and status of the last run, without the tracks."""
        counts = np.zeros(max(n_events, 1), np.uint32)
        first = np.zeros(max(n_events, 1), np.uint64)
        status = np.zeros(max(n_events, 1), np.uint32)
        self._check(self._lib.velo_fetch(self._h, None, 0, _p(counts), _p(first), _p(status)), "velo_fetch")
        return counts[:n_events], first[:n_events], status[:n_events]

    def fetch_into(self, tracks: np.ndarray, counts: np.ndarray, first: np.ndarray, status: np.ndarray):
        self._check(self._lib.velo_fetch(self._h, _p(tracks), len(tracks), _p(counts), _p(first),
                                         _p(status)), "velo_fetch")

    def search_packed_into(self, buf, offsets, sizes, options, tracks, counts, first, status):
        st = self._lib.velo_search_packed(self._h, buf.ctypes.data, _p(offsets), _p(sizes), len(offsets),
                                          ctypes.byref(options), _p(tracks), len(tracks), _p(counts),
                                          _p(first), _p(status))
        self._check(st, "velo_search_packed")

    def time_runs(self, options: Optional[Options] = None, warmup: int = 3, iters: int = 10,
                  flush_l2: bool = True) -> float:
        opts = options or default_options()
        ms = ctypes.c_float()
        self._check(self._lib.velo_time_runs(self._h, ctypes.byref(opts), warmup, iters, int(flush_l2),
                                             ctypes.byref(ms)), "velo_time_runs")
        return float(ms.value)

    def autotune(self, base: Optional[Options] = None, iters: int = 3):
        """Fastest launch configuration for the staged events: (Options, ms)."""
        b = base or default_options()
        best = Options()
        ms = ctypes.c_float()
        self._check(self._lib.velo_autotune(self._h, ctypes.byref(b), iters, ctypes.byref(best), ctypes.byref(ms)),
                    "velo_autotune")
        return best, float(ms.value)

    def set_mlp(self, weights: np.ndarray, keep_threshold: float, window_margin: float, min_keep_rate: float,
                max_event_hits: int = 0):
        w = np.ascontiguousarray(weights, np.float32)
        assert w.size == MLP_PARAMS
        self._check(self._lib.velo_set_mlp(self._h, _p(w), keep_threshold, window_margin, min_keep_rate,
                                           int(max_event_hits)), "velo_set_mlp")

    def dump_doublets(self, capacity: int, keep_one_in: int = 1, options: Optional[Options] = None):
        """Features and {event, h0, h1} of sampled doublets of a plain run on the staged events."""
        feats = np.zeros((max(capacity, 1), MLP_INPUTS), np.float32)
        ids = np.zeros((max(capacity, 1), 3), np.uint32)
        count = ctypes.c_uint64()
        opts = options or default_options()
        self._check(self._lib.velo_dump_doublets(self._h, ctypes.byref(opts), keep_one_in, _p(feats), _p(ids),
                                                 capacity, ctypes.byref(count)), "velo_dump_doublets")
        k = min(int(count.value), capacity)
        return feats[:k], ids[:k], int(count.value)

    def fit_tracks(self, capacity: int) -> np.ndarray:
        """Straight-line fits of the last run's tracks, in fetch order."""
        fits = np.zeros(max(capacity, 1), FIT_DTYPE)
        self._check(self._lib.velo_fit_tracks(self._h, _p(fits), capacity), "velo_fit_tracks")
        return fits

    def sort_staged(self):
        """The reference's per-module x-sort, on the device, of the staged events."""
        self._check(self._lib.velo_sort_staged(self._h), "velo_sort_staged")

    def fetch_staged(self, nbytes: int) -> np.ndarray:
        buf = np.zeros(max(nbytes, 1), np.uint8)
        self._check(self._lib.velo_fetch_staged(self._h, _p(buf), nbytes), "velo_fetch_staged")
        return buf[:nbytes]

    def search_unsorted(self, blobs: Sequence[bytes], options: Optional[Options] = None):
        """Sort on the device, then search: (tracks per event, status, x-sorted blobs)."""
        from .events import pack_events
        buf, offs, sizes = pack_events(blobs)
        self.stage(buf, offs, sizes)
        self.sort_staged()
        self.run(options or default_options())
        cap = int(sum(max(int(np.frombuffer(b[4:8], "<i4")[0]), 1) if len(b) >= 8 else 1 for b in blobs))
        tracks, counts, first, status = self.fetch(len(blobs), cap)
        staged = self.fetch_staged(int(offs[-1] + sizes[-1]) if len(blobs) else 0)
        sorted_blobs = [staged[int(o):int(o) + int(n)].tobytes() for o, n in zip(offs, sizes)]
        per = [tracks[int(first[e]):int(first[e]) + int(counts[e])] for e in range(len(blobs))]
        return per, status, sorted_blobs

    def stats(self) -> Stats:
        s = Stats()
        self._check(self._lib.velo_get_stats(self._h, ctypes.byref(s)), "velo_get_stats")
        return s

    def synchronize(self):
        self._check(self._lib.velo_synchronize(self._h), "velo_synchronize")

    def host_alloc(self, nbytes: int) -> np.ndarray:
        """Pinned host buffer (uint8 array); freed by :meth:`host_free`."""
        p = ctypes.c_void_p()
        self._check(self._lib.velo_host_alloc(self._h, nbytes, ctypes.byref(p)), "velo_host_alloc")
        arr = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p.value))
        return arr

    def host_free(self, arr: np.ndarray):
        self._check(self._lib.velo_host_free(self._h, ctypes.c_void_p(arr.ctypes.data)), "velo_host_free")


API_BENCH_PATH = os.path.join(PKG, "_build", "libvelo_api_bench.so")


def reference_api_times(blobs: Sequence[bytes], entry: str, warmup: int, steps: int, want_sorted: bool = False):
    """Host wall-clock milliseconds of `steps` calls of a reference-signature
    entry point on std::vector<std::vector<uint8_t> > input (the timing
    harness libvelo_api_bench.so): entry "independent_execute" (unsorted
    events; sort and search) or "gpuPixelSearchByTriplet" (x-sorted events).
    Returns (ms per call, tracks of the last call, each event's output
    digest as validation.event_hashes computes it, the input bytes after the
    last call or None).  The entry points
    print what the reference prints; that text goes to this process's
    stdout, so callers that own stdout redirect it around the call."""
    load()
    if not os.path.exists(API_BENCH_PATH):
        raise RuntimeError(f"timing harness missing: {API_BENCH_PATH}; run cl_forward_gb300.build.build()")
    lib = ctypes.CDLL(API_BENCH_PATH)
    vp = ctypes.c_void_p
    lib.velo_bench_reference_api.argtypes = [vp, vp, vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_int32, vp, vp, vp, vp]
    n = len(blobs)
    sizes = np.array([len(b) for b in blobs], np.uint64)
    offs = np.zeros(n, np.uint64)
    if n:
        offs[1:] = np.cumsum(sizes)[:-1]
    buf = np.frombuffer(b"".join(blobs), np.uint8) if n else np.zeros(1, np.uint8)
    ms = np.zeros(max(steps, 1), np.float64)
    tracks = ctypes.c_uint64()
    digests = np.zeros(max(n, 1), np.uint64)
    out = np.zeros(max(int(sizes.sum()), 1), np.uint8) if want_sorted else None
    code = {"independent_execute": 0, "gpuPixelSearchByTriplet": 1}[entry]
    st = lib.velo_bench_reference_api(buf.ctypes.data, _p(offs), _p(sizes), n, code, warmup, steps, _p(ms),
                                      ctypes.byref(tracks), _p(digests),
                                      _p(out) if out is not None else None)
    if st != 0:
        raise RuntimeError("velo_bench_reference_api: bad arguments")
    sorted_blobs = None
    if out is not None:
        sorted_blobs = [out[int(o):int(o) + int(z)].tobytes() for o, z in zip(offs, sizes)]
    return ms[:steps].copy(), int(tracks.value), digests[:n].copy(), sorted_blobs


def _check_free(st: int, what: str):
    if st != OK:
        raise VeloError(st, f"{what}: {load().velo_status_string(st).decode()}")


def mlp_train(x: np.ndarray, label: np.ndarray, target: np.ndarray, weights: np.ndarray, steps: int,
              batch: int = 4096, lr: float = 1e-3, seed: int = 0):
    """Adam training with the library's CUDA kernels; returns (weights, loss per step)."""
    x = np.ascontiguousarray(x, np.float32)
    label = np.ascontiguousarray(label, np.float32)
    target = np.ascontiguousarray(target, np.float32)
    w = np.ascontiguousarray(weights, np.float32).copy()
    loss = np.zeros(steps, np.float32)
    _check_free(load().velo_mlp_train(_p(x), _p(label), _p(target), len(x), steps, batch, lr, seed, _p(w), _p(loss)),
                "velo_mlp_train")
    return w, loss


def mlp_grad(weights: np.ndarray, x: np.ndarray, label: np.ndarray, target: np.ndarray):
    w = np.ascontiguousarray(weights, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    label = np.ascontiguousarray(label, np.float32)
    target = np.ascontiguousarray(target, np.float32)
    g = np.zeros(MLP_PARAMS, np.float32)
    loss = ctypes.c_float()
    _check_free(load().velo_mlp_grad(_p(w), _p(x), _p(label), _p(target), len(x), _p(g), ctypes.byref(loss)),
                "velo_mlp_grad")
    return g, float(loss.value)


def mlp_forward(weights: np.ndarray, x: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(weights, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((len(x), 2), np.float32)
    _check_free(load().velo_mlp_forward(_p(w), _p(x), len(x), _p(out)), "velo_mlp_forward")
    return out
