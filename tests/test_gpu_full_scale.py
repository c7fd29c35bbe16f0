"""The batched configuration at its full size (100,000 uneven events), where
the oracle would take minutes: size-independent properties instead.

* the device sort equals the reference's host sort (a sample of events);
* an order-independent checksum of every event's tracks is the same for three
  launch configurations (persistent 64-thread, one 256-thread CTA per event,
  persistent 128-thread with the other register build);
* every track is well formed: 3-24 hits, all inside its event, distinct, in
  strictly descending module order; no event is flagged invalid.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_EVENTS = 100_000


def _tracks_in_event_order(ctx, n):
    """Tracks of the last run grouped by event, with per-event counts."""
    counts, _, _ = ctx.fetch_counts(n)
    total = int(counts.sum())
    from cl_forward_gb300 import events
    tracks = np.zeros(max(total, 1), events.TRACK_DTYPE)
    c2 = np.zeros(n, np.uint32)
    f2 = np.zeros(n, np.uint64)
    s2 = np.zeros(n, np.uint32)
    ctx.fetch_into(tracks, c2, f2, s2)
    assert np.array_equal(c2, counts)
    starts = np.concatenate([[0], np.cumsum(counts.astype(np.int64))[:-1]])
    idx = np.repeat(f2.astype(np.int64) - starts, counts.astype(np.int64)) + np.arange(total, dtype=np.int64)
    words = tracks.view(np.uint32).reshape(-1, 25)[:total][idx]
    return words, counts.astype(np.int64), starts, s2


def _event_checksums(words, counts, starts):
    """Sum over each event's tracks of a hash of the whole 100-byte record."""
    w = words.astype(np.uint64)
    h = np.zeros(len(w), np.uint64)
    for k in range(25):
        h = h * np.uint64(1000003) + w[:, k]
    out = np.zeros(len(counts), np.uint64)
    nz = counts > 0
    out[nz] = np.add.reduceat(h, starts[nz])
    return out


def test_batched_100k_properties(gpu_ctx):
    from cl_forward_gb300 import events, generator, native
    raw, _ = generator.generate_parallel(range(2_000_000, 2_000_000 + N_EVENTS), generator.CONFIG_BATCHED)
    buf, offs, sizes = events.pack_events(raw)
    gpu_ctx.stage(buf, offs, sizes)
    gpu_ctx.sort_staged()
    sorted_buf = gpu_ctx.fetch_staged(len(buf))
    for e in range(0, N_EVENTS, 997):                        # the device sort is the reference's
        a, m = int(offs[e]), int(sizes[e])
        assert bytes(sorted_buf[a:a + m]) == native.sort_by_x(raw[e])
    H = np.array([int(np.frombuffer(b[4:8], "<i4")[0]) for b in raw], np.int64)
    sums = []
    for opts in (native.default_options(),
                 native.default_options(launch_mode=0, threads_per_event=256, register_ctas=5, smem_hits=0),
                 native.default_options(threads_per_event=128, register_ctas=4)):
        gpu_ctx.stage(sorted_buf, offs, sizes)
        gpu_ctx.run(opts)
        words, counts, starts, status = _tracks_in_event_order(gpu_ctx, N_EVENTS)
        assert not np.any(status & native.EVENT_INVALID)
        sums.append(_event_checksums(words, counts, starts))
    assert np.array_equal(sums[0], sums[1]) and np.array_equal(sums[0], sums[2])
    assert counts.sum() > 100 * N_EVENTS
    # well-formed tracks (the last run)
    nh = words[:, 0].astype(np.int64)
    assert nh.min() >= 3 and nh.max() <= 24
    hits = words[:, 1:].astype(np.int64)
    valid = np.arange(24)[None, :] < nh[:, None]
    ev_of = np.repeat(np.arange(N_EVENTS), counts)
    assert np.all(np.where(valid, hits, 0) < H[ev_of][:, None])
    assert np.all(np.where(valid, hits, 0) >= 0)
    s = np.sort(np.where(valid, hits, -1 - np.arange(24)[None, :]), axis=1)
    assert np.all(np.diff(s, axis=1) != 0)                   # distinct hits
    # descending module order, on the first 5,000 events' tracks
    lim = int(counts[:5000].sum())
    mod_of = []
    base = 0
    for e in range(5000):
        ev = events.unpack_event(bytes(sorted_buf[int(offs[e]):int(offs[e]) + int(sizes[e])]))
        mod_of.append(np.repeat(np.arange(len(ev.hit_num)), ev.hit_num))
    mods = np.concatenate(mod_of)
    hit_base = np.concatenate([[0], np.cumsum(H[:5000])[:-1]])
    g = np.where(valid[:lim], hits[:lim] + hit_base[ev_of[:lim]][:, None], 0)
    m = mods[g]
    later = np.arange(1, 24)[None, :] < nh[:lim, None]
    assert np.all(np.where(later, m[:, 1:] < m[:, :-1], True))
