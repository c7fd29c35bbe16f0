"""Event layout, .dat container, generator determinism and truth encoding."""
import os

import numpy as np

from cl_forward_gb300 import events, fuzz, generator


def test_pack_unpack_roundtrip():
    ev, _ = generator.generate_event(3)
    blob = events.pack_event(ev)
    assert len(blob) == events.event_nbytes(ev.n_sensors, ev.n_hits)
    back = events.unpack_event(blob)
    for f in ("sensor_z", "hit_start", "hit_num", "hit_id", "x", "y", "z"):
        assert np.array_equal(getattr(ev, f), getattr(back, f))
    assert events.pack_event(back) == blob


def test_generator_is_seeded_and_batched_equals_single():
    a = [events.pack_event(generator.generate_event(s)[0]) for s in (5, 6, 7)]
    b, _ = generator.generate([5, 6, 7])
    assert a == b
    c, _ = generator.generate([6])
    assert c[0] == a[1]


def test_geometry_and_ids():
    blob, truth = generator.generate([11])
    ev = events.unpack_event(blob[0])
    assert ev.n_sensors == 52
    assert np.all(np.diff(ev.sensor_z) > 0)
    mod = ev.module_of_hit()
    assert np.array_equal(ev.hit_id & 0xFF, mod.astype(np.uint32))
    assert np.all(ev.z == generator.MODULE_Z[mod].astype(np.float32))
    # left modules (even) hold x < 0.5, right (odd) x > -0.5
    left = (mod % 2) == 0
    assert np.all(ev.x[left] < 0.5 + 0.1) and np.all(ev.x[~left] > -0.5 - 0.1)
    r = np.hypot(ev.x, ev.y)
    assert r.min() > 5.0 and r.max() < 42.1
    keys = ev.hit_id >> 8
    real = keys < generator.NOISE_KEY_BASE
    counts = np.bincount(keys[real] - 1, minlength=len(truth[0].p))
    assert np.array_equal(counts, truth[0].n_hits)


def test_config_sizes():
    small = [events.unpack_event(b).n_hits for b in generator.generate(range(30))[0]]
    dense = [events.unpack_event(b).n_hits for b in generator.generate(range(10), generator.CONFIG_STRESS)[0]]
    assert 300 < np.mean(small) < 3000
    assert np.mean(dense) > 2.5 * np.mean(small)


def test_dat_roundtrip(tmp_path):
    blob = generator.generate([2])[0][0]
    p = os.path.join(tmp_path, "0.dat")
    events.write_dat(p, blob)
    with open(p, "ab") as f:
        f.write(b"\x01\x02trailing bytes the driver ignores")
    assert events.read_dat(p) == blob


def test_fuzz_events_are_valid_layouts():
    for s in range(20):
        ev = events.unpack_event(fuzz.fuzz_event(s, n_modules=3 + s % 50))
        assert int(ev.hit_num.sum()) == ev.n_hits
        assert np.array_equal(ev.hit_start, np.concatenate([[0], np.cumsum(ev.hit_num)[:-1]]).astype(np.int32))


def test_pack_events_alignment():
    blobs = generator.generate(range(5))[0]
    buf, offs, sizes = events.pack_events(blobs)
    assert np.all(offs % 16 == 0)
    assert list(events.iter_blobs(buf, offs, sizes)) == blobs
