"""Truth matching and the order-independent comparator."""
import numpy as np

from cl_forward_gb300 import events, generator, validation


def _track(idx):
    t = np.zeros(1, events.TRACK_DTYPE)
    t["hitsNum"] = len(idx)
    t["hits"][0, :len(idx)] = idx
    return t


def _event(keys_per_hit):
    n = len(keys_per_hit)
    ids = np.array([(k << 8) | (i % 52) for i, k in enumerate(keys_per_hit)], np.uint32)
    ev = events.Event(np.zeros(1, np.int32), np.zeros(1, np.int32), np.array([n], np.int32), ids,
                      np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32))
    return events.pack_event(ev)


def test_rates_hand_made():
    # particle 1: hits 0-3, particle 2: hits 4-6, particle 3: 7-9 (unfound), noise hit 10
    keys = [1, 1, 1, 1, 2, 2, 2, 3, 3, 3, generator.NOISE_KEY_BASE]
    blob = _event(keys)
    truth = generator.Truth(p=np.array([1.0, 5.0, 3.0]), eta=np.zeros(3), n_hits=np.array([4, 3, 3]))
    tracks = np.concatenate([_track([0, 1, 2, 3]),      # P1
                             _track([0, 1, 2]),         # P1 clone
                             _track([4, 5, 6]),         # P2
                             _track([4, 7, 10])])       # ghost (33 % purity)
    r = validation.event_rates(tracks, blob, truth)
    assert r.reconstructible == 3 and r.matched == 2
    assert r.ghosts == 1 and r.clones == 1 and r.tracks == 4
    assert abs(r.efficiency - 2 / 3) < 1e-12
    assert abs(r.ghost_rate - 0.25) < 1e-12
    assert abs(r.clone_rate - 1 / 3) < 1e-12
    assert r.recon_low == 1 and r.matched_low == 1 and r.matched_high == 1


def test_purity_threshold():
    keys = [1, 1, 1, 1, 1, 1, 1, 2, 2, 2]
    blob = _event(keys)
    truth = generator.Truth(p=np.array([3.0, 3.0]), eta=np.zeros(2), n_hits=np.array([7, 3]))
    ok = validation.event_rates(_track([0, 1, 2, 3, 4, 5, 6, 7, 8, 9]), blob, truth)   # 70 %: matched
    assert ok.ghosts == 0 and ok.matched == 1
    bad = validation.event_rates(_track([0, 1, 7, 8, 2]), blob, truth)               # 60 %: ghost
    assert bad.ghosts == 1


def test_compare_events_order_independent():
    blob = _event([1, 1, 1, 2, 2, 2])
    a = np.concatenate([_track([0, 1, 2]), _track([3, 4, 5])])
    b = np.concatenate([_track([5, 4, 3]), _track([2, 0, 1])])
    assert validation.compare_events([a], [b], [blob]) == []
    c = np.concatenate([_track([0, 1, 2]), _track([3, 4])])
    assert validation.compare_events([a], [c], [blob]) == [0]


def test_fast_rates_equal_reference_rates():
    from oracle import oracle
    blobs, truths = generator.generate(range(40))
    sb = [oracle.sort_by_x(b) for b in blobs]
    tracks, _ = oracle.search(sb, 4)
    slow = validation.rates(tracks, sb, truths)
    fast = validation.rates_fast(tracks, sb, truths)
    assert slow == fast


def test_packed_helpers_equal_per_event_forms():
    """The whole-batch forms used at 100,000 events (packed sort, chunked
    restatement, digests, rates) equal the per-event ones."""
    from oracle import oracle
    blobs, truths = generator.generate(range(60), generator.CONFIG_BATCHED)
    buf, offs, sizes = events.pack_events(blobs)
    sbuf = oracle.sort_packed(buf, offs, sizes)
    sb = [oracle.sort_by_x(b) for b in blobs]
    assert [bytes(sbuf[int(o):int(o) + int(s)]) for o, s in zip(offs, sizes)] == sb
    words, counts, status = oracle.search_packed(sbuf, offs, sizes, chunk=7)
    tracks, st = oracle.search(sb, 4)
    assert np.array_equal(status, st)
    assert counts.tolist() == [len(t) for t in tracks]
    assert np.array_equal(words, np.concatenate([t.view(np.uint32).reshape(-1, 25) for t in tracks]))
    ids, base = validation.hit_ids_packed(sbuf, offs)
    fast = validation.rates_packed(words, counts, ids, base, truths)
    assert fast == validation.rates(tracks, sb, truths)
    sub = np.arange(0, 60, 3)
    assert validation.rates_packed(words, counts, ids, base, truths, events=sub) == \
        validation.rates([tracks[e] for e in sub], [sb[e] for e in sub], [truths[e] for e in sub])
    # digests: order-independent within an event, sensitive to any word
    h = validation.event_hashes(words, counts)
    perm = []
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    for e in range(60):
        perm.extend((starts[e] + np.random.default_rng(e).permutation(counts[e])).tolist())
    assert np.array_equal(validation.event_hashes(words[perm], counts), h)
    w2 = words.copy()
    w2[int(starts[5]), 3] ^= 1
    h2 = validation.event_hashes(w2, counts)
    assert h2[5] != h[5] and np.array_equal(np.delete(h2, 5), np.delete(h, 5))
    assert len(set(h.tolist())) == 60
