"""The track-dump comparison (reference printTrack format), on oracle output."""
import os

import numpy as np


def test_dumps_round_trip_and_compare(tmp_path, oracle_lib):
    from cl_forward_gb300 import compare, events, generator
    blobs = [oracle_lib.sort_by_x(b) for b in generator.generate(range(20, 26))[0]]
    tracks, _ = oracle_lib.search(blobs, 4)
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    for e, blob in enumerate(blobs):
        compare.write_dump(str(a / f"{e}.out"), blob, tracks[e])
        # the other side lists its tracks in reverse order: still identical
        compare.write_dump(str(b / f"{e}.out"), blob, tracks[e][::-1])
    ev0 = events.unpack_event(blobs[0])
    got = compare.read_dump(str(a / "0.out"))
    want = [tuple(int(ev0.hit_id[h]) for h in t["hits"][:int(t["hitsNum"])]) for t in tracks[0]]
    assert got == want
    res = compare.compare_dirs(str(a), str(b))
    assert res["total"]["identical_events"] == len(blobs) and res["total"]["only_a"] == 0
    assert compare.main([str(a), str(b), "--quiet"]) == 0
    # drop one hit of one track and one whole track on side B of event 1
    t1 = tracks[1].copy()
    t1[0]["hitsNum"] -= 1
    compare.write_dump(str(b / "1.out"), blobs[1], t1[:-1])
    r = compare.compare_dirs(str(a), str(b))["events"][1]
    assert r["only_a"] == 2 and r["only_b"] == 1
    assert any(p["only_b"] == [] and len(p["only_a"]) == 1 for p in r["same_first_hit"])
    assert compare.main([str(a), str(b), "--quiet"]) == 1
