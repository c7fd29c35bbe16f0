"""Event-buffer layout of the VELO search-by-triplet input and output.

One event is one contiguous little-endian blob, the layout parsed by
``setHPointersFromInput`` (Tools.cpp:68-80) and re-derived inside the kernel
(Kernel.cl:612-624)::

    int32   number_of_sensors  (S)
    int32   number_of_hits     (H)
    int32   sensor_Zs[S]
    int32   sensor_hitStarts[S]
    int32   sensor_hitNums[S]
    uint32  hit_IDs[H]
    float32 hit_Xs[H]
    float32 hit_Ys[H]
    float32 hit_Zs[H]

Output per event is an array of ``Track {uint32 hitsNum; uint32 hits[24];}``
(100 bytes, KernelDefinitions.h:59-62); each ``hits`` entry is an
event-local index into the (x-sorted) hit arrays.

The ``.dat`` container read by the standalone driver
(IndependentEntrypoint.cpp:89-123) is ``int32 nameLen; char name[nameLen];
int32 dataSize; uint8 data[dataSize]`` followed by bytes the driver ignores.
"""
from __future__ import annotations

import dataclasses
import struct
from typing import Iterable, List, Sequence

import numpy as np

MAX_TRACK_SIZE = 24       # KernelDefinitions.h:16
MAX_TRACKS = 3000         # KernelDefinitions.h:15
TTF_MODULO = 2000         # KernelDefinitions.h:23
TRACK_DTYPE = np.dtype([("hitsNum", "<u4"), ("hits", "<u4", (MAX_TRACK_SIZE,))])
assert TRACK_DTYPE.itemsize == 100


@dataclasses.dataclass
class Event:
    """A parsed view of one event blob (arrays are copies, not views)."""

    sensor_z: np.ndarray        # int32[S]
    hit_start: np.ndarray       # int32[S]
    hit_num: np.ndarray         # int32[S]
    hit_id: np.ndarray          # uint32[H]
    x: np.ndarray               # float32[H]
    y: np.ndarray               # float32[H]
    z: np.ndarray               # float32[H]

    @property
    def n_sensors(self) -> int:
        return int(self.sensor_z.shape[0])

    @property
    def n_hits(self) -> int:
        return int(self.hit_id.shape[0])

    def module_of_hit(self) -> np.ndarray:
        """Module index of every hit (hits are contiguous per module)."""
        out = np.full(self.n_hits, -1, np.int32)
        for m in range(self.n_sensors):
            s, n = int(self.hit_start[m]), int(self.hit_num[m])
            out[s:s + n] = m
        return out


def event_nbytes(n_sensors: int, n_hits: int) -> int:
    return 8 + 12 * n_sensors + 16 * n_hits


def pack_event(ev: Event) -> bytes:
    """Serialise an :class:`Event` to the blob layout above."""
    S, H = ev.n_sensors, ev.n_hits
    parts = [
        struct.pack("<ii", S, H),
        np.ascontiguousarray(ev.sensor_z, "<i4").tobytes(),
        np.ascontiguousarray(ev.hit_start, "<i4").tobytes(),
        np.ascontiguousarray(ev.hit_num, "<i4").tobytes(),
        np.ascontiguousarray(ev.hit_id, "<u4").tobytes(),
        np.ascontiguousarray(ev.x, "<f4").tobytes(),
        np.ascontiguousarray(ev.y, "<f4").tobytes(),
        np.ascontiguousarray(ev.z, "<f4").tobytes(),
    ]
    blob = b"".join(parts)
    assert len(blob) == event_nbytes(S, H)
    return blob


def unpack_event(blob) -> Event:
    """Parse a blob (bytes / bytearray / uint8 array) into an :class:`Event`."""
    buf = memoryview(bytes(blob)) if not isinstance(blob, (bytes, bytearray)) else memoryview(blob)
    if len(buf) < 8:
        raise ValueError("event blob shorter than its 8-byte header")
    S, H = struct.unpack_from("<ii", buf, 0)
    if S < 0 or H < 0 or len(buf) < event_nbytes(S, H):
        raise ValueError(f"event blob of {len(buf)} bytes does not hold S={S}, H={H}")
    o = 8
    sz = np.frombuffer(buf, "<i4", S, o).copy(); o += 4 * S
    st = np.frombuffer(buf, "<i4", S, o).copy(); o += 4 * S
    nm = np.frombuffer(buf, "<i4", S, o).copy(); o += 4 * S
    ids = np.frombuffer(buf, "<u4", H, o).copy(); o += 4 * H
    x = np.frombuffer(buf, "<f4", H, o).copy(); o += 4 * H
    y = np.frombuffer(buf, "<f4", H, o).copy(); o += 4 * H
    z = np.frombuffer(buf, "<f4", H, o).copy()
    return Event(sz, st, nm, ids, x, y, z)


def read_dat(path: str) -> bytes:
    """Read the event blob of one ``.dat`` file (IndependentEntrypoint.cpp:89-123)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 4:
        raise ValueError(f"{path}: too short for a .dat header")
    (name_len,) = struct.unpack_from("<i", data, 0)
    o = 4 + name_len
    if name_len < 0 or len(data) < o + 4:
        raise ValueError(f"{path}: bad name length {name_len}")
    (size,) = struct.unpack_from("<i", data, o)
    o += 4
    if size < 0 or len(data) < o + size:
        raise ValueError(f"{path}: data size {size} exceeds the file")
    return data[o:o + size]


def write_dat(path: str, blob: bytes, name: bytes = b"PrPixelCudaHandler") -> None:
    """Write one event blob in the ``.dat`` container the driver reads."""
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(name)))
        f.write(name)
        f.write(struct.pack("<i", len(blob)))
        f.write(blob)


def tracks_from_bytes(buf) -> np.ndarray:
    """View ``count * 100`` output bytes as a structured Track array."""
    arr = np.frombuffer(bytes(buf), dtype=TRACK_DTYPE)
    return arr


def track_id_sets(tracks: np.ndarray, hit_ids: np.ndarray) -> List[tuple]:
    """Map each track's hit indices to hit IDs, as a sorted tuple per track.

    The result is the order-independent form used for parity: the multiset of
    tracks, each track the sorted tuple of its hit IDs.
    """
    out = []
    for t in tracks:
        n = int(t["hitsNum"])
        out.append(tuple(sorted(int(hit_ids[h]) for h in t["hits"][:n])))
    out.sort()
    return out


def pack_events(blobs: Sequence[bytes], align: int = 16):
    """Concatenate blobs with each start aligned to ``align`` bytes.

    Returns ``(buffer uint8[...], offsets uint64[n], sizes uint64[n])``.
    """
    sizes = np.array([len(b) for b in blobs], dtype=np.uint64)
    offsets = np.zeros(len(blobs), dtype=np.uint64)
    total = 0
    for i, s in enumerate(sizes):
        offsets[i] = total
        total += (int(s) + align - 1) // align * align
    buf = np.zeros(max(total, align), dtype=np.uint8)
    for i, b in enumerate(blobs):
        o = int(offsets[i])
        buf[o:o + len(b)] = np.frombuffer(b, dtype=np.uint8)
    return buf, offsets, sizes


def iter_blobs(buf: np.ndarray, offsets: Iterable[int], sizes: Iterable[int]):
    for o, s in zip(offsets, sizes):
        yield bytes(buf[int(o):int(o) + int(s)])
