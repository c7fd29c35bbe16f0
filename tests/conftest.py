import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_tracks.npz")
GOLDEN_SETS = ("velo", "fuzz", "mcdata", "edge")
GOLDEN_Y = (1, 2, 4)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _split(buf, offs, sizes):
    return [bytes(buf[int(o):int(o) + int(s)]) for o, s in zip(offs, sizes)]


@pytest.fixture(scope="session")
def golden():
    """{set: {"input": [...], "sorted": [...], "tracks": {Y: [np.uint32 (n,25) per event]}}}"""
    z = np.load(GOLDEN)
    out = {}
    for name in GOLDEN_SETS:
        d = {"input": _split(z[f"{name}_input"], z[f"{name}_input_off"], z[f"{name}_input_size"]),
             "sorted": _split(z[f"{name}_sorted"], z[f"{name}_sorted_off"], z[f"{name}_sorted_size"]),
             "tracks": {}}
        for Y in GOLDEN_Y:
            flat, counts = z[f"{name}_tracks_y{Y}"], z[f"{name}_counts_y{Y}"]
            cuts = np.concatenate([[0], np.cumsum(counts)])
            d["tracks"][Y] = [flat[cuts[i]:cuts[i + 1]] for i in range(len(counts))]
        out[name] = d
    return out


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def native_lib():
    from cl_forward_gb300 import build, native
    build.build()
    return native.load()


@pytest.fixture(scope="session")
def gpu_ctx(native_lib):
    from cl_forward_gb300 import native
    ctx = native.Context(0)
    yield ctx
    ctx.close()


def index_lists_words(words):
    """Sorted hit-index tuples from (n, 25) uint32 Track words."""
    out = [tuple(int(h) for h in w[1:1 + int(w[0])]) for w in words]
    out.sort()
    return out


def index_lists(tracks):
    """Sorted hit-index tuples from a TRACK_DTYPE array."""
    out = [tuple(int(h) for h in t["hits"][:int(t["hitsNum"])]) for t in tracks]
    out.sort()
    return out
