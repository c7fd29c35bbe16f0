"""ctypes front-end to the CPU oracle (TEST INFRASTRUCTURE ONLY).

``liboracle`` is the C restatement in velo_oracle.c (built here and on any
machine by :func:`build`); ``libref_emu`` is the reference's own kernel under
the work-group emulator (oracle/_ref, built by build_ref.py only where the
reference sources exist).  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time
from typing import List, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libvelo_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_emu.so")

TRACK_DTYPE = np.dtype([("hitsNum", "<u4"), ("hits", "<u4", (24,))])

EVENT_RING_OVERFLOW = 0x1
EVENT_TRACK_OVERFLOW = 0x2
EVENT_MAX_TRACKS = 0x4
EVENT_INVALID = 0x8
EVENT_DEGENERATE = 0x10
PARITY_EXCLUDING = EVENT_RING_OVERFLOW | EVENT_TRACK_OVERFLOW | EVENT_MAX_TRACKS | EVENT_DEGENERATE

CFLAGS = ["-O3", "-std=gnu11", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


class Counters(ctypes.Structure):
    _fields_ = [("window_evals", ctypes.c_uint64), ("forward_fits", ctypes.c_uint64),
                ("seed_fits", ctypes.c_uint64), ("seed_scatters", ctypes.c_uint64)]


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "velo_oracle.c"), os.path.join(HERE, "velo_oracle.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in src)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run(["gcc", *CFLAGS, "-shared", "-o", tmp, src[0], "-lpthread", "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        build()
        l = ctypes.CDLL(LIB)
        l.vo_validate_event.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        l.vo_sort_by_x.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        l.vo_search_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.POINTER(Counters)]
        _lib = l
    return _lib


def ref_available() -> bool:
    if os.path.exists(REF_LIB):
        return True
    try:
        from . import build_ref  # type: ignore
    except ImportError:
        import importlib.util
        spec = importlib.util.spec_from_file_location("build_ref", os.path.join(HERE, "build_ref.py"))
        build_ref = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(build_ref)
    return build_ref.build(quiet=True) is not None


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference emulator not built (reference sources absent)")
        l = ctypes.CDLL(REF_LIB)
        l.ref_search_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        l.ref_preorder_by_x.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _ref = l
    return _ref


def ref_sort_by_x(blobs: Sequence[bytes]) -> List[bytes]:
    """The reference's own preorder_by_x (Tools.cpp:46-66) over a batch of events."""
    bufs = [ctypes.create_string_buffer(bytes(b), len(b)) for b in blobs]
    ptrs = (ctypes.c_void_p * len(bufs))(*[ctypes.addressof(b) for b in bufs])
    sizes = np.array([len(b) for b in blobs], np.uint64)
    if ref_lib().ref_preorder_by_x(ptrs, _ptr(sizes), len(blobs)) != 0:
        raise RuntimeError("reference preorder_by_x failed")
    return [b.raw for b in bufs]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def sort_by_x(blob: bytes) -> bytes:
    """The reference's per-module x-sort (Tools.cpp:46-66) of one event."""
    buf = np.frombuffer(bytearray(blob), dtype=np.uint8).copy()
    if lib().vo_sort_by_x(_ptr(buf), len(blob)) != 0:
        raise ValueError("invalid event blob")
    return buf.tobytes()


def _pack(blobs: Sequence[bytes]):
    sizes = np.array([len(b) for b in blobs], np.uint64)
    offsets = np.zeros(len(blobs), np.uint64)
    if len(blobs):
        offsets[1:] = np.cumsum(sizes)[:-1]
    buf = np.frombuffer(b"".join(blobs) + b"\0" * 16, dtype=np.uint8).copy()
    n_hits = np.array([int(np.frombuffer(b[4:8], "<i4")[0]) if len(b) >= 8 else 0 for b in blobs],
                      np.int64)
    return buf, offsets, sizes, n_hits


def search(blobs: Sequence[bytes], y_lanes: int = 4, threads: int = 0, counters: bool = False):
    """Run the restatement on x-sorted events.

    Returns ``(tracks: list of TRACK_DTYPE arrays, status uint32[n][, Counters])``.
    """
    buf, offsets, sizes, n_hits = _pack(blobs)
    n = len(blobs)
    cap = np.maximum(n_hits, 1).astype(np.uint32)
    first = np.zeros(n, np.uint64)
    if n:
        first[1:] = np.cumsum(cap.astype(np.uint64))[:-1]
    out = np.zeros(int(cap.sum()) + 1, TRACK_DTYPE)
    counts = np.zeros(n, np.uint32)
    status = np.zeros(n, np.uint32)
    c = Counters()
    lib().vo_search_batch(_ptr(buf), _ptr(offsets), _ptr(sizes), n, y_lanes, threads, _ptr(out),
                          _ptr(first), _ptr(cap), _ptr(counts), _ptr(status), ctypes.byref(c))
    tracks = [out[int(first[e]):int(first[e]) + int(counts[e])].copy() for e in range(n)]
    if counters:
        return tracks, status, c
    return tracks, status


def packed_hit_counts(buf: np.ndarray, offsets: np.ndarray) -> np.ndarray:
    """H of every event of a packed batch (the int32 at byte 4 of each blob)."""
    idx = offsets.astype(np.int64)[:, None] + np.arange(4, 8)[None, :]
    return np.ascontiguousarray(buf[idx.ravel()]).view("<i4").astype(np.int64)


def sort_packed(buf: np.ndarray, offsets: np.ndarray, sizes: np.ndarray) -> np.ndarray:
    """The reference's per-module x-sort (Tools.cpp:46-66) of every event of a
    packed batch; returns a sorted copy (same offsets)."""
    out = np.array(buf, dtype=np.uint8, copy=True)
    base = out.ctypes.data
    f = lib().vo_sort_by_x
    for o, s in zip(offsets.tolist(), sizes.tolist()):
        if f(ctypes.c_void_p(base + o), s) != 0:
            raise ValueError(f"invalid event blob at offset {o}")
    return out


def search_packed(buf: np.ndarray, offsets: np.ndarray, sizes: np.ndarray, y_lanes: int = 4,
                  threads: int = 0, chunk: int = 4000):
    """Restatement over a packed batch of x-sorted events, ``chunk`` events per
    call to bound memory.

    Returns ``(words, counts, status)``: ``words`` the (T, 25) uint32 Track
    records of all events, event by event; ``counts`` int64[n]; ``status``
    uint32[n].  Per-event Python objects are never made, so 100,000-event
    batches stay cheap.
    """
    n = len(offsets)
    H = packed_hit_counts(buf, offsets)
    counts = np.zeros(n, np.uint32)
    status = np.zeros(n, np.uint32)
    parts = []
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        cap = np.maximum(H[a:b], 1).astype(np.uint32)
        first = np.zeros(b - a, np.uint64)
        first[1:] = np.cumsum(cap.astype(np.uint64))[:-1]
        out = np.zeros(int(cap.sum()) + 1, TRACK_DTYPE)
        off = np.ascontiguousarray(offsets[a:b], np.uint64)
        siz = np.ascontiguousarray(sizes[a:b], np.uint64)
        c = np.zeros(b - a, np.uint32)
        s = np.zeros(b - a, np.uint32)
        lib().vo_search_batch(_ptr(buf), _ptr(off), _ptr(siz), b - a, y_lanes, threads, _ptr(out),
                              _ptr(first), _ptr(cap), _ptr(c), _ptr(s), None)
        c64 = c.astype(np.int64)
        starts = np.concatenate([[0], np.cumsum(c64)[:-1]])
        idx = np.repeat(first.astype(np.int64) - starts, c64) + np.arange(int(c64.sum()), dtype=np.int64)
        parts.append(out.view(np.uint32).reshape(-1, 25)[idx].copy())
        counts[a:b] = c
        status[a:b] = s
        del out
    words = np.concatenate(parts) if parts else np.zeros((0, 25), np.uint32)
    return words, counts.astype(np.int64), status


def time_search(blobs: Sequence[bytes], y_lanes: int = 4, threads: int = 0) -> float:
    """Wall seconds of one multi-threaded oracle pass over ``blobs`` (packing excluded)."""
    buf, offsets, sizes, n_hits = _pack(blobs)
    n = len(blobs)
    cap = np.maximum(n_hits, 1).astype(np.uint32)
    first = np.zeros(n, np.uint64)
    if n:
        first[1:] = np.cumsum(cap.astype(np.uint64))[:-1]
    out = np.zeros(int(cap.sum()) + 1, TRACK_DTYPE)
    counts = np.zeros(n, np.uint32)
    status = np.zeros(n, np.uint32)
    t0 = time.perf_counter()
    lib().vo_search_batch(_ptr(buf), _ptr(offsets), _ptr(sizes), n, y_lanes, threads, _ptr(out),
                          _ptr(first), _ptr(cap), _ptr(counts), _ptr(status), None)
    return time.perf_counter() - t0


def ref_search(blobs: Sequence[bytes], y_lanes: int = 4, threads: int = 0, sched_seed: int = 0):
    """Run the reference kernel itself (emulated work-groups) on x-sorted events."""
    buf, offsets, sizes, n_hits = _pack(blobs)
    n = len(blobs)
    cap = np.minimum(np.maximum(n_hits, 1), 3000).astype(np.uint32)
    first = np.zeros(n, np.uint64)
    if n:
        first[1:] = np.cumsum(cap.astype(np.uint64))[:-1]
    out = np.zeros(int(cap.sum()) + 1, TRACK_DTYPE)
    counts = np.zeros(n, np.uint32)
    nh = n_hits.astype(np.int32)
    rc = ref_lib().ref_search_batch(_ptr(buf), _ptr(offsets), _ptr(nh), n, y_lanes, threads,
                                    sched_seed, _ptr(out), _ptr(first), _ptr(cap), _ptr(counts))
    if rc != 0:
        raise RuntimeError(f"reference emulator failed: {rc}")
    return [out[int(first[e]):int(first[e]) + min(int(counts[e]), int(cap[e]))].copy()
            for e in range(n)]


def id_sets(tracks: np.ndarray, blob: bytes) -> List[Tuple[int, ...]]:
    """Order-independent parity form: sorted list of per-track sorted hit-ID tuples."""
    S, H = np.frombuffer(blob[:8], "<i4")
    ids = np.frombuffer(blob, "<u4", int(H), 8 + 12 * int(S))
    out = [tuple(sorted(int(ids[h]) for h in t["hits"][:int(t["hitsNum"])])) for t in tracks]
    out.sort()
    return out


def index_lists(tracks: np.ndarray) -> List[Tuple[int, ...]]:
    """Sorted list of per-track hit-index tuples in emitted order."""
    out = [tuple(int(h) for h in t["hits"][:int(t["hitsNum"])]) for t in tracks]
    out.sort()
    return out
