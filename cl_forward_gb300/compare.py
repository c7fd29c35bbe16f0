"""Compare two sets of track dumps in the reference's printTrack format.

The reference's standalone driver writes ``results/<i>.out`` per event
(format of KernelInvoker.cpp:285-306: ``Track #k, length n`` then one line per
hit ``<id> (<index>) module <m>, x <x>, y <y>, z <z>``); so does this
project's driver (``clpixel ... --dump DIR``).  Dumps from two producers are
compared event by event on hit IDs, which do not depend on how each producer
ordered the hits before searching:

* a track matches when the other side has a track with the same set of hit
  IDs (the order-independent comparison the parity tests use);
* tracks without a match are paired by their first hit ID where possible and
  reported with the hit IDs each side has that the other lacks.

    python -m cl_forward_gb300.compare DIR_A DIR_B [--events N] [--quiet]
"""
from __future__ import annotations

import argparse
import os
import re
import sys
from collections import Counter
from typing import Dict, List, Sequence, Tuple

_TRACK = re.compile(r"^Track #(\d+), length (\d+)\s*$")
_HIT = re.compile(r"^\s*(\d+) \((\d+)\) module\s+(-?\d+),")


def read_dump(path: str) -> List[Tuple[int, ...]]:
    """Tracks of one dump file, each the tuple of its hit IDs in dump order."""
    tracks: List[Tuple[int, ...]] = []
    cur: List[int] = []
    want = -1
    with open(path) as f:
        for line in f:
            m = _TRACK.match(line)
            if m:
                if want >= 0:
                    tracks.append(tuple(cur))
                cur, want = [], int(m.group(2))
                continue
            h = _HIT.match(line)
            if h and want >= 0:
                cur.append(int(h.group(1)))
    if want >= 0:
        tracks.append(tuple(cur))
    for t in tracks:
        if len(t) < 1:
            raise ValueError(f"{path}: a track without hits")
    return tracks


def write_dump(path: str, blob: bytes, tracks) -> None:
    """Write tracks (a Track array of one event) in the printTrack format."""
    import numpy as np
    from .events import unpack_event
    ev = unpack_event(blob)
    zmod = {int(z): m for m, z in enumerate(ev.sensor_z)}
    with open(path, "w") as f:
        for i, t in enumerate(tracks):
            n = int(t["hitsNum"])
            f.write(f"Track #{i}, length {n}\n")
            for h in t["hits"][:n]:
                h = int(h)
                m = zmod.get(int(np.float32(ev.z[h])), -1)
                f.write(f" {int(ev.hit_id[h]):8d} ({h}) module {m:2d}, x {ev.x[h]:6g}, y {ev.y[h]:6g}, "
                        f"z {ev.z[h]:6g}\n")
            f.write("\n")


def compare_event(a: Sequence[Tuple[int, ...]], b: Sequence[Tuple[int, ...]]) -> Dict[str, object]:
    """Matched / unmatched tracks of one event, compared as sets of hit IDs."""
    ka = Counter(tuple(sorted(t)) for t in a)
    kb = Counter(tuple(sorted(t)) for t in b)
    only_a = list((ka - kb).elements())
    only_b = list((kb - ka).elements())
    by_first_b = {}
    for t in b:
        if tuple(sorted(t)) in set(only_b):
            by_first_b.setdefault(t[0], t)
    pairs = []
    for t in a:
        if tuple(sorted(t)) in set(only_a) and t[0] in by_first_b:
            u = by_first_b[t[0]]
            pairs.append({"first_hit": t[0], "only_a": sorted(set(t) - set(u)), "only_b": sorted(set(u) - set(t))})
    return {"tracks_a": len(a), "tracks_b": len(b), "matched": sum((ka & kb).values()),
            "only_a": len(only_a), "only_b": len(only_b), "same_first_hit": pairs}


def compare_dirs(dir_a: str, dir_b: str, n_events: int = 0) -> Dict[str, object]:
    names = sorted((f for f in os.listdir(dir_a) if f.endswith(".out")), key=lambda f: int(f.split(".")[0]))
    if n_events:
        names = names[:n_events]
    events, tot = [], Counter()
    for name in names:
        pb = os.path.join(dir_b, name)
        if not os.path.exists(pb):
            raise FileNotFoundError(pb)
        r = compare_event(read_dump(os.path.join(dir_a, name)), read_dump(pb))
        r["event"] = int(name.split(".")[0])
        events.append(r)
        for k in ("tracks_a", "tracks_b", "matched", "only_a", "only_b"):
            tot[k] += r[k]
    tot["events"] = len(events)
    tot["identical_events"] = sum(1 for r in events if r["only_a"] == 0 and r["only_b"] == 0)
    return {"total": dict(tot), "events": events}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("dir_a")
    ap.add_argument("dir_b")
    ap.add_argument("--events", type=int, default=0, help="compare only the first N events")
    ap.add_argument("--quiet", action="store_true", help="print the totals only")
    a = ap.parse_args(argv)
    res = compare_dirs(a.dir_a, a.dir_b, a.events)
    if not a.quiet:
        for r in res["events"]:
            if r["only_a"] or r["only_b"]:
                print(f"event {r['event']}: {r['matched']} matched, {r['only_a']} only in A, "
                      f"{r['only_b']} only in B")
                for p in r["same_first_hit"]:
                    print(f"  first hit {p['first_hit']}: A has {p['only_a']}, B has {p['only_b']}")
    t = res["total"]
    print(f"{t['events']} events, {t['identical_events']} identical; {t['matched']} tracks matched, "
          f"{t['only_a']} only in A, {t['only_b']} only in B")
    return 0 if t["only_a"] == 0 and t["only_b"] == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
