"""Python mirror of the reference's host entry points, on the C ABI.

Same names and argument meaning as GpuPixelSearchByTriplet.h:12-29,
KernelInvoker.h:27-31 and Tools.h:47 of dcampora/cl_forward:

* ``input``  -- a list of event blobs (``bytes``; ``bytearray`` or uint8 numpy
  arrays where the call sorts in place);
* ``output`` -- a list that receives, per event, ``count * 100`` bytes of
  ``Track {uint32 hitsNum; uint32 hits[24];}`` records.

Where the reference ends the process on an error (exit(-1), Tools.h:27-34),
these raise :class:`cl_forward_gb300.native.VeloError`.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, MutableSequence, Sequence

import numpy as np

from . import native
from .events import TRACK_DTYPE

MAX_EVENTS_PER_KERNEL = 16000   # GpuPixelSearchByTriplet.cpp:53

_ctx = None
verbosity = 0


def context() -> native.Context:
    """The process-wide context (device ``$VELO_DEVICE``, default 0)."""
    global _ctx
    if _ctx is None:
        _ctx = native.Context(int(os.environ.get("VELO_DEVICE", "0")))
    return _ctx


def _as_bytes(ev) -> bytes:
    if isinstance(ev, np.ndarray):
        return ev.tobytes()
    return bytes(ev)


def preorder_by_x(input: Sequence) -> None:
    """Sort each module's hits by x, in place (Tools.cpp:46-66)."""
    lib = native.load()
    for ev in input:
        if isinstance(ev, bytes):
            raise TypeError("preorder_by_x sorts in place: pass bytearray or numpy uint8 buffers")
        if isinstance(ev, np.ndarray):
            ptr, n = ev.ctypes.data, ev.nbytes
        else:
            if len(ev) == 0:
                continue
            ptr, n = ctypes.addressof((ctypes.c_char * len(ev)).from_buffer(ev)), len(ev)
        st = lib.velo_sort_by_x(ptr, n)
        if st != native.OK:
            raise native.VeloError(st, "preorder_by_x: invalid event blob")


def invokeParallelSearch(startingEvent: int, eventsToProcess: int, input: Sequence,
                         output: MutableSequence) -> int:
    """Search input[startingEvent:+eventsToProcess] (KernelInvoker.cpp:14-275)."""
    if eventsToProcess <= 0:
        return 0
    blobs = [_as_bytes(input[startingEvent + i]) for i in range(eventsToProcess)]
    tracks, _ = context().search(blobs, native.default_options())
    for i, t in enumerate(tracks):
        output[startingEvent + i] = t.tobytes()
    return 0


def gpuPixelSearchByTripletInvocation(input: Sequence, output: List) -> int:
    """Resize output and search in chunks of 16000 events (GpuPixelSearchByTriplet.cpp:44-65)."""
    output[:] = [b""] * len(input)
    for i in range(0, len(input), MAX_EVENTS_PER_KERNEL):
        n = min(len(input) - i, MAX_EVENTS_PER_KERNEL)
        invokeParallelSearch(i, n, input, output)
    return 0


def gpuPixelSearchByTriplet(input: Sequence, output: List) -> int:
    """Framework entry: input already x-sorted; silent (GpuPixelSearchByTriplet.cpp:29-37)."""
    global verbosity
    verbosity = 0
    return gpuPixelSearchByTripletInvocation(input, output)


def independent_execute(input: Sequence, output: List) -> int:
    """Standalone entry: x-sort in place, then search (GpuPixelSearchByTriplet.cpp:4-22).

    As in the library's C++ entry point, the sort runs on the GPU with the
    reference's permutation (velo_sort_search), in chunks of 16000 events,
    and leaves the input buffers sorted."""
    global verbosity
    verbosity = 3
    for ev in input:
        if isinstance(ev, bytes):
            raise TypeError("independent_execute sorts in place: pass bytearray or numpy uint8 buffers")
    output[:] = [b""] * len(input)
    for i in range(0, len(input), MAX_EVENTS_PER_KERNEL):
        chunk = list(input[i:i + MAX_EVENTS_PER_KERNEL])
        tracks, _ = context().sort_search(chunk, native.default_options(host_direct=1))
        for k, t in enumerate(tracks):
            output[i + k] = t.tobytes()
    return 0


def independent_post_execute(output: Sequence) -> None:
    if verbosity >= 3:
        print(f"\nSize of output: {len(output)} entries")


def tracks_of(output_entry: bytes) -> np.ndarray:
    """View one output entry as a Track array."""
    return np.frombuffer(output_entry, TRACK_DTYPE)
