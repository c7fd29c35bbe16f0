"""Order-independent track comparison and truth-matched tracking rates.

Parity form (both sides of every parity test): per event, the sorted list of
tracks, each track the sorted tuple of its hit IDs.  The reference's own diff
tool (tools/comparetracks.py:13-77) matches tracks by first hit ID only; this
compares whole hit sets and multiplicities.

Tracking rates (the reference has no checker; the same one is applied to the
oracle and to the GPU output): a track is matched to particle P if at least
70 % of its hits carry P's key (``hit_id >> 8`` in the synthetic events).  A
particle is reconstructible with at least 3 recorded hits.  Efficiency =
matched reconstructible particles / reconstructible; ghost rate = unmatched
tracks / tracks; clone rate = extra tracks matched to an already matched
particle / matched tracks.  Rates are also split at p = 2 GeV.
"""
from __future__ import annotations

import dataclasses
from collections import Counter
from typing import Dict, Iterable, List, Sequence, Tuple

import numpy as np

from .events import unpack_event
from .generator import NOISE_KEY_BASE, Truth

PURITY = 0.7


def id_lists(tracks: np.ndarray, blob: bytes) -> List[Tuple[int, ...]]:
    ev = unpack_event(blob)
    out = []
    for t in tracks:
        n = int(t["hitsNum"])
        out.append(tuple(sorted(int(ev.hit_id[h]) for h in t["hits"][:n])))
    out.sort()
    return out


def compare_events(a_tracks: Sequence[np.ndarray], b_tracks: Sequence[np.ndarray],
                   blobs: Sequence[bytes]) -> List[int]:
    """Indices of events whose track multisets (as hit-ID sets) differ."""
    bad = []
    for e, (a, b) in enumerate(zip(a_tracks, b_tracks)):
        if len(a) != len(b) or id_lists(a, blobs[e]) != id_lists(b, blobs[e]):
            bad.append(e)
    return bad


@dataclasses.dataclass
class Rates:
    reconstructible: int = 0
    matched: int = 0
    tracks: int = 0
    ghosts: int = 0
    clones: int = 0
    recon_low: int = 0
    matched_low: int = 0
    recon_high: int = 0
    matched_high: int = 0

    def add(self, o: "Rates") -> None:
        for f in dataclasses.fields(self):
            setattr(self, f.name, getattr(self, f.name) + getattr(o, f.name))

    @property
    def efficiency(self) -> float:
        return self.matched / self.reconstructible if self.reconstructible else 0.0

    @property
    def ghost_rate(self) -> float:
        return self.ghosts / self.tracks if self.tracks else 0.0

    @property
    def clone_rate(self) -> float:
        m = self.tracks - self.ghosts
        return self.clones / m if m else 0.0

    @property
    def efficiency_low_p(self) -> float:
        return self.matched_low / self.recon_low if self.recon_low else 0.0

    @property
    def efficiency_high_p(self) -> float:
        return self.matched_high / self.recon_high if self.recon_high else 0.0

    def as_dict(self) -> Dict[str, float]:
        return {"efficiency": self.efficiency, "ghost_rate": self.ghost_rate,
                "clone_rate": self.clone_rate, "efficiency_p_lt_2": self.efficiency_low_p,
                "efficiency_p_ge_2": self.efficiency_high_p, "tracks": self.tracks,
                "reconstructible": self.reconstructible}


def event_rates(tracks: np.ndarray, blob: bytes, truth: Truth, min_hits: int = 3) -> Rates:
    ev = unpack_event(blob)
    keys = ev.hit_id >> np.uint32(8)
    r = Rates()
    recon = truth.n_hits >= min_hits
    r.reconstructible = int(recon.sum())
    low = truth.p < 2.0
    r.recon_low = int((recon & low).sum())
    r.recon_high = int((recon & ~low).sum())
    found = Counter()
    for t in tracks:
        n = int(t["hitsNum"])
        r.tracks += 1
        ks = Counter(int(keys[h]) for h in t["hits"][:n])
        key, cnt = ks.most_common(1)[0]
        if key >= NOISE_KEY_BASE or cnt < PURITY * n:
            r.ghosts += 1
            continue
        found[key] += 1
    for key, cnt in found.items():
        i = key - 1
        if cnt > 1:
            r.clones += cnt - 1
        if 0 <= i < len(recon) and recon[i]:
            r.matched += 1
            if low[i]:
                r.matched_low += 1
            else:
                r.matched_high += 1
    return r


def rates(all_tracks: Iterable[np.ndarray], blobs: Sequence[bytes], truths: Sequence[Truth]) -> Rates:
    total = Rates()
    for t, b, tr in zip(all_tracks, blobs, truths):
        total.add(event_rates(t, b, tr))
    return total


def event_rates_fast(tracks: np.ndarray, hit_id: np.ndarray, truth: Truth, min_hits: int = 3) -> Rates:
    """Vectorised :func:`event_rates` (same definitions), for large batches."""
    r = Rates()
    recon = truth.n_hits >= min_hits
    low = truth.p < 2.0
    r.reconstructible = int(recon.sum())
    r.recon_low = int((recon & low).sum())
    r.recon_high = int((recon & ~low).sum())
    T = len(tracks)
    r.tracks = T
    if T == 0:
        return r
    n = tracks["hitsNum"].astype(np.int64)
    hits = tracks["hits"].astype(np.int64)
    mask = np.arange(hits.shape[1])[None, :] < n[:, None]
    keys = (hit_id[np.where(mask, hits, 0)] >> np.uint32(8)).astype(np.int64)
    keys = np.where(mask, keys, -1)
    # majority key per track: compare every slot against every slot
    eq = (keys[:, :, None] == keys[:, None, :]) & mask[:, None, :]
    cnt = eq.sum(axis=2)
    best = np.argmax(np.where(mask, cnt, -1), axis=1)
    top_key = keys[np.arange(T), best]
    top_cnt = cnt[np.arange(T), best]
    matched = (top_key < NOISE_KEY_BASE) & (top_cnt >= PURITY * n)
    r.ghosts = int((~matched).sum())
    mk = top_key[matched]
    if len(mk):
        uniq, mult = np.unique(mk, return_counts=True)
        r.clones = int((mult - 1).sum())
        idx = uniq - 1
        ok = (idx >= 0) & (idx < len(recon))
        idx = idx[ok]
        good = recon[idx]
        r.matched = int(good.sum())
        r.matched_low = int((good & low[idx]).sum())
        r.matched_high = int((good & ~low[idx]).sum())
    return r


def rates_fast(all_tracks, blobs: Sequence[bytes], truths: Sequence[Truth]) -> Rates:
    total = Rates()
    for t, b, tr in zip(all_tracks, blobs, truths):
        S, H = np.frombuffer(b[:8], "<i4")
        ids = np.frombuffer(b, "<u4", int(H), 8 + 12 * int(S))
        total.add(event_rates_fast(t, ids, tr))
    return total
