"""Generate tests/golden/golden_tracks.npz from the reference itself.

Expected outputs come from the reference's own code, compiled from the
reference checkout by oracle/build_ref.py: the per-module x-sort is the
reference's preorder_by_x (Tools.cpp:46-66) and the tracks are the
reference's clSearchByTriplets (Kernel.cl:597-816) run under the work-group
emulator (oracle/ref_emu.c), at local size (64, Y).  Inputs are seeded
synthetic events (cl_forward_gb300.generator / .fuzz), stored as bytes so the
fixture does not depend on the generator staying bit-identical, and the
first six real events of the reference's mcdata/ (real geometry: several z
values per module, unsorted hits).

Run in a checkout next to the reference sources:
    python tests/golden/make_golden.py [--reference DIR]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cl_forward_gb300 import events, fuzz, generator  # noqa: E402
from oracle import build_ref, oracle  # noqa: E402

OUT = os.path.join(HERE, "golden_tracks.npz")
Y_VALUES = (1, 2, 4)


def _concat(blobs):
    sizes = np.array([len(b) for b in blobs], np.int64)
    offs = np.zeros(len(blobs), np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    return np.frombuffer(b"".join(blobs), np.uint8).copy(), offs, sizes


def _tracks_flat(track_lists):
    counts = np.array([len(t) for t in track_lists], np.int64)
    flat = np.concatenate([t.view(np.uint32).reshape(-1, 25) for t in track_lists]) if counts.sum() else \
        np.zeros((0, 25), np.uint32)
    return flat, counts


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    if a.reference:
        os.environ["CL_FORWARD_REFERENCE"] = a.reference
    if not oracle.ref_available():
        sys.exit("reference sources not available: cannot build oracle/_ref")
    sets = {
        "velo": generator.generate(range(4))[0],
        "fuzz": [fuzz.fuzz_event(5000 + s, max_per_module=20, grid=1.0, lines=10, x_span=45)
                 for s in (0, 3, 7, 11, 19, 23, 42, 57)]
                + [fuzz.fuzz_event(2000 + s, jitter_z=True) for s in range(4)]
                + [fuzz.fuzz_event(s, grid=2.0) for s in range(4)],
        "mcdata": [events.read_dat(os.path.join(build_ref.default_reference(), "mcdata", f"{i}.dat"))
                   for i in range(6)],
        "edge": [fuzz.empty_event(), fuzz.empty_event(0), fuzz.empty_event(4),
                 fuzz.fuzz_event(3000, n_modules=5), fuzz.fuzz_event(3001, n_modules=7),
                 fuzz.fuzz_event(3002, max_per_module=1, lines=1)],
    }
    arrays = {}
    for name, blobs in sets.items():
        sorted_blobs = oracle.ref_sort_by_x(blobs)
        _, status = oracle.search(sorted_blobs, 4)
        keep = [i for i in range(len(blobs)) if not (status[i] & oracle.PARITY_EXCLUDING)]
        blobs = [blobs[i] for i in keep]
        sorted_blobs = [sorted_blobs[i] for i in keep]
        buf, offs, sizes = _concat(blobs)
        arrays[f"{name}_input"], arrays[f"{name}_input_off"], arrays[f"{name}_input_size"] = buf, offs, sizes
        buf, offs, sizes = _concat(sorted_blobs)
        arrays[f"{name}_sorted"], arrays[f"{name}_sorted_off"], arrays[f"{name}_sorted_size"] = buf, offs, sizes
        for Y in Y_VALUES:
            ref = oracle.ref_search(sorted_blobs, Y, sched_seed=Y)
            flat, counts = _tracks_flat(ref)
            arrays[f"{name}_tracks_y{Y}"] = flat
            arrays[f"{name}_counts_y{Y}"] = counts
        print(f"{name}: {len(blobs)} events, tracks at Y=4: {int(arrays[f'{name}_counts_y4'].sum())}")
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
