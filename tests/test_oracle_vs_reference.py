"""The oracle restatement against the reference kernel run here (fresh seeds).

Needs the reference sources (oracle/_ref is built from them); skipped elsewhere.
"""
import glob
import os

import numpy as np
import pytest

from conftest import index_lists

from oracle.build_ref import default_reference  # noqa: E402

ref_dir = default_reference()


@pytest.fixture(scope="module")
def ref(oracle_lib):
    if not oracle_lib.ref_available():
        pytest.skip("reference sources not present")
    return oracle_lib


def _compare(ref, blobs, y, seed):
    sb = ref.ref_sort_by_x(blobs)
    tracks, status = ref.search(sb, y)
    keep = [i for i in range(len(sb)) if not (status[i] & ref.PARITY_EXCLUDING)]
    got = ref.ref_search([sb[i] for i in keep], y, sched_seed=seed)
    bad = [i for j, i in enumerate(keep) if index_lists(tracks[i]) != index_lists(got[j])]
    return bad, len(keep)


def test_velo_events(ref):
    from cl_forward_gb300 import generator
    blobs, _ = generator.generate(range(200, 240))
    bad, n = _compare(ref, blobs, 4, 99)
    assert n == 40 and not bad


def test_schedule_seeds_agree(ref):
    """The reference kernel's track contents do not depend on the order in
    which its work-items run between barriers: the in-order schedule and five
    seeded random schedules all give the restatement's tracks."""
    from cl_forward_gb300 import generator
    blobs, _ = generator.generate(range(1000, 1030))
    for seed in range(6):
        bad, n = _compare(ref, blobs, 4, seed)
        assert n == 30 and not bad, (seed, bad)


@pytest.mark.parametrize("y", [1, 3, 4, 16])
def test_fuzz_events(ref, y):
    from cl_forward_gb300 import fuzz
    blobs = [fuzz.fuzz_event(7000 + s, max_per_module=20, grid=1.0, lines=10, x_span=45) for s in range(60)]
    blobs += [fuzz.fuzz_event(8000 + s, jitter_z=True) for s in range(20)]
    bad, n = _compare(ref, blobs, y, y)
    assert n > 50 and not bad


def test_uneven_and_dense_events(ref):
    from cl_forward_gb300 import generator
    blobs = generator.generate(range(300, 310), generator.CONFIG_STRESS)[0]
    blobs += generator.generate(range(400, 420), generator.CONFIG_BATCHED)[0]
    bad, n = _compare(ref, blobs, 4, 5)
    assert n >= 25 and not bad


def test_reference_mcdata(ref):
    from cl_forward_gb300 import events
    files = sorted(glob.glob(os.path.join(ref_dir, "mcdata", "*.dat")))
    if not files:
        pytest.skip("mcdata not present")
    blobs = [events.read_dat(f) for f in files]
    sb = ref.ref_sort_by_x(blobs)
    assert [ref.sort_by_x(b) for b in blobs] == sb
    bad, n = _compare(ref, blobs, 4, 1)
    assert n == len(files) and not bad


def test_overflow_flags(oracle_lib):
    from cl_forward_gb300 import fuzz
    # long straight lines on one side give tracks of more than 24 hits
    blobs = [oracle_lib.sort_by_x(fuzz.fuzz_event(s, lines=12, max_per_module=2)) for s in range(40)]
    _, status = oracle_lib.search(blobs, 4)
    assert np.any(status & oracle_lib.EVENT_TRACK_OVERFLOW)


def test_predecessor_tracks_in_mcdata_are_found(oracle_lib):
    """Each mcdata file carries, after the event, the tracks of a predecessor
    producer (records {4-word header, hitsNum, hits[24]}, hit indices in the
    file's unsorted order).  They are not this kernel's output, but the same
    physics: the restatement (pinned to the reference kernel) reproduces at
    least 95 % of them exactly as sets of hit IDs (measured: 96.0 %)."""
    import struct
    from cl_forward_gb300 import events
    mc = os.path.join(ref_dir, "mcdata")
    if not os.path.isdir(mc):
        pytest.skip("reference mcdata not available")
    total = exact = 0
    for name in sorted(os.listdir(mc), key=lambda f: int(f.split(".")[0])):
        data = open(os.path.join(mc, name), "rb").read()
        (nl,) = struct.unpack_from("<i", data, 0)
        o = 4 + nl
        (size,) = struct.unpack_from("<i", data, o)
        blob = data[o + 4:o + 4 + size]
        o += 4 + size
        (nbytes,) = struct.unpack_from("<i", data, o)
        rec = np.frombuffer(data, np.uint32, nbytes // 4, o + 4).reshape(-1, 29)
        ev = events.unpack_event(blob)
        sb = oracle_lib.sort_by_x(blob)
        evs = events.unpack_event(sb)
        tracks, _ = oracle_lib.search([sb], 4)
        mine = {frozenset(int(evs.hit_id[h]) for h in t["hits"][:int(t["hitsNum"])]) for t in tracks[0]}
        for r in rec:
            n = int(r[4])
            if n >= 3 and np.all(r[5:5 + n] < len(ev.hit_id)):
                total += 1
                exact += frozenset(int(ev.hit_id[h]) for h in r[5:5 + n]) in mine
    assert total > 15000 and exact >= 0.95 * total
