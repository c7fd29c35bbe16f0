"""The oracle restatement against golden vectors produced by the reference itself.

tests/golden/golden_tracks.npz holds seeded events, the reference's own
preorder_by_x output for them, and the tracks of the reference's own kernel at
local sizes (64, Y) for Y = 1, 2, 4 (see tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from conftest import GOLDEN_SETS, GOLDEN_Y, index_lists, index_lists_words


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_oracle_sort_matches_reference_sort(golden, oracle_lib, name):
    for raw, ref_sorted in zip(golden[name]["input"], golden[name]["sorted"]):
        assert oracle_lib.sort_by_x(raw) == ref_sorted


@pytest.mark.parametrize("name", GOLDEN_SETS)
@pytest.mark.parametrize("y", GOLDEN_Y)
def test_oracle_tracks_match_reference(golden, oracle_lib, name, y):
    tracks, status = oracle_lib.search(golden[name]["sorted"], y)
    assert not np.any(status & oracle_lib.PARITY_EXCLUDING)
    for e, (mine, ref) in enumerate(zip(tracks, golden[name]["tracks"][y])):
        assert index_lists(mine) == index_lists_words(ref), f"{name} event {e}"


def test_golden_tracks_are_whole_records(golden):
    # unused hit slots of the reference's Track records are zero
    for name in GOLDEN_SETS:
        for words in golden[name]["tracks"][4]:
            for w in words:
                n = int(w[0])
                assert 3 <= n <= 24
                assert not np.any(w[1 + n:])


def test_golden_covers_y_dependence(golden):
    # at least one golden event resolves a tie differently at Y=1 and Y=4
    diff = sum(index_lists_words(a) != index_lists_words(b)
               for a, b in zip(golden["fuzz"]["tracks"][1], golden["fuzz"]["tracks"][4]))
    assert diff >= 1
