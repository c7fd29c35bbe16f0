"""Wide pinning sweep of the restatement against the reference kernel run here.

7,000+ events on seeds no other test uses: config-2 physics events (Y = 4,
seeded work-item schedules), uneven and dense events, and adversarial fuzz
events at Y = 1, 2, 3, 4, 5, 7, 8, 16.  About a minute on 8 cores.  Needs the
reference sources (oracle/_ref is built from them); skipped elsewhere.
"""
import pytest

from conftest import index_lists


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
    return len(keep), bad


@pytest.mark.parametrize("part", range(10))
def test_physics_events(ref, part):
    from cl_forward_gb300 import generator
    blobs, _ = generator.generate_parallel(range(20000 + 500 * part, 20500 + 500 * part))
    n, bad = _compare(ref, blobs, 4, 100 + part)
    assert n >= 495 and not bad, bad[:10]


def test_uneven_and_stress_events(ref):
    from cl_forward_gb300 import generator
    for params, seeds in ((generator.CONFIG_BATCHED, range(30000, 30300)),
                          (generator.CONFIG_STRESS, range(31000, 31100))):
        blobs, _ = generator.generate_parallel(seeds, params)
        n, bad = _compare(ref, blobs, 4, 7)
        assert n >= len(blobs) - 5 and not bad, bad[:10]


@pytest.mark.parametrize("y", [1, 2, 3, 4, 5, 7, 8, 16])
def test_fuzz_events(ref, y):
    from cl_forward_gb300 import fuzz
    blobs = [fuzz.fuzz_event(40000 + 1000 * y + s, max_per_module=20, grid=1.0, lines=10, x_span=45)
             for s in range(150)]
    blobs += [fuzz.fuzz_event(60000 + 1000 * y + s, jitter_z=True) for s in range(50)]
    blobs += [fuzz.fuzz_event(80000 + 1000 * y + s, grid=2.0) for s in range(50)]
    n, bad = _compare(ref, blobs, y, y)
    assert n > 200 and not bad, bad[:10]
