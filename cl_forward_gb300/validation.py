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


_HASH_MUL = np.array([(0x9E3779B97F4A7C15 * (2 * k + 1)) & 0xFFFFFFFFFFFFFFFF for k in range(25)],
                     np.uint64)


def event_hashes(words: np.ndarray, counts: np.ndarray) -> np.ndarray:
    """Order-independent digest of each event's tracks: the sum (mod 2**64) over
    its tracks of a 64-bit hash of the whole 100-byte record.  Equal digests
    mean equal track multisets (as hit-index lists in emitted order, zeros
    past hitsNum) up to a 2**-64 collision.  ``words`` is (T, 25) uint32,
    event by event; ``counts`` the tracks per event."""
    counts = np.asarray(counts, np.int64)
    out = np.zeros(len(counts), np.uint64)
    if len(words) == 0:
        return out
    h = np.zeros(len(words), np.uint64)
    with np.errstate(over="ignore"):
        for k in range(25):
            x = (words[:, k].astype(np.uint64) + np.uint64(k + 1)) * _HASH_MUL[k]
            x ^= x >> np.uint64(29)
            h = (h ^ x) * np.uint64(0xBF58476D1CE4E5B9)
            h ^= h >> np.uint64(31)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    nz = counts > 0
    with np.errstate(over="ignore"):
        out[nz] = np.add.reduceat(h, starts[nz])
    return out


def hit_ids_packed(buf: np.ndarray, offsets: np.ndarray):
    """Hit IDs of every event of a packed batch, concatenated, and each
    event's first position in that array."""
    parts = []
    for o in offsets.tolist():
        S, H = np.frombuffer(buf, "<i4", 2, o)
        parts.append(np.frombuffer(buf, "<u4", int(H), o + 8 + 12 * int(S)))
    ids = np.concatenate(parts) if parts else np.zeros(0, np.uint32)
    lens = np.array([len(p) for p in parts], np.int64)
    return ids, np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)


def rates_packed(words: np.ndarray, counts: np.ndarray, hit_ids: np.ndarray, hit_base: np.ndarray,
                 truths: Sequence[Truth], events: np.ndarray = None, min_hits: int = 3) -> Rates:
    """:func:`rates` over a whole batch at once (same definitions).

    ``words``/``counts`` as in :func:`event_hashes`; ``hit_ids``/``hit_base``
    from :func:`hit_ids_packed`; ``events`` optionally restricts the rates to
    a subset of event indices.  A track's majority key is the median of its
    sorted hit keys: a key holding at least 70 % of the hits holds the middle
    position, so the median is the only candidate the purity cut can accept.
    """
    n = len(counts)
    counts = np.asarray(counts, np.int64)
    sel = np.ones(n, bool) if events is None else np.isin(np.arange(n), events)
    r = Rates()
    nh_parts, p_parts, pbase = [], [], [0]
    for t in truths:
        nh_parts.append(np.asarray(t.n_hits))
        p_parts.append(np.asarray(t.p))
        pbase.append(pbase[-1] + len(t.n_hits))
    nh = np.concatenate(nh_parts) if nh_parts else np.zeros(0, np.int64)
    pp = np.concatenate(p_parts) if p_parts else np.zeros(0)
    pbase = np.array(pbase, np.int64)
    ev_of_particle = np.repeat(np.arange(n), np.diff(pbase))
    recon = (nh >= min_hits) & sel[ev_of_particle]
    low = pp < 2.0
    r.reconstructible = int(recon.sum())
    r.recon_low = int((recon & low).sum())
    r.recon_high = int((recon & ~low).sum())
    ev_of = np.repeat(np.arange(n), counts)
    keep = sel[ev_of]
    w = words[keep]
    ev_of = ev_of[keep]
    T = len(w)
    r.tracks = T
    if T == 0:
        return r
    nhit = w[:, 0].astype(np.int64)
    mask = np.arange(24)[None, :] < nhit[:, None]
    g = np.where(mask, w[:, 1:].astype(np.int64) + hit_base[ev_of][:, None], 0)
    keys = np.where(mask, (hit_ids[g] >> np.uint32(8)).astype(np.int64), np.iinfo(np.int64).max)
    keys.sort(axis=1)
    med = keys[np.arange(T), nhit // 2]
    cnt = (keys == med[:, None]).sum(axis=1)
    matched = (med < NOISE_KEY_BASE) & (cnt >= PURITY * nhit)
    r.ghosts = int((~matched).sum())
    gk = ev_of[matched] * (1 << 32) + med[matched]
    if len(gk):
        uniq, mult = np.unique(gk, return_counts=True)
        r.clones = int((mult - 1).sum())
        e = uniq >> 32
        k = (uniq & 0xFFFFFFFF) - 1
        ok = (k >= 0) & (k < np.diff(pbase)[e])
        pi = pbase[e[ok]] + k[ok]
        good = recon[pi]
        r.matched = int(good.sum())
        r.matched_low = int((good & low[pi]).sum())
        r.matched_high = int((good & ~low[pi]).sum())
    return r


def rates_fast(all_tracks, blobs: Sequence[bytes], truths: Sequence[Truth]) -> Rates:
    total = Rates()
    for t, b, tr in zip(all_tracks, blobs, truths):
        S, H = np.frombuffer(b[:8], "<i4")
        ids = np.frombuffer(b, "<u4", int(H), 8 + 12 * int(S))
        total.add(event_rates_fast(t, ids, tr))
    return total
