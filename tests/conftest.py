import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


DYNAMIC_PREFIX = "arrivals"   # fixtures with a changing population (per-snapshot ids)


def golden_names():
    """Fixtures of a fixed population (ids, positions per snapshot)."""
    return sorted(n for n in (os.path.splitext(os.path.basename(p))[0]
                              for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
                  if not n.startswith(DYNAMIC_PREFIX))


def dynamic_golden_names():
    """Fixtures with timed insertion and remove-at-goal."""
    return sorted(n for n in (os.path.splitext(os.path.basename(p))[0]
                              for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
                  if n.startswith(DYNAMIC_PREFIX))


def dynamic_snapshots(g):
    """[(step, ids, positions)] of a dynamic fixture, in the reference's list order."""
    off = g["snap_off"]
    return [(int(s), g["snap_ids"][off[k]:off[k + 1]], g["snap_pos"][off[k]:off[k + 1]])
            for k, s in enumerate(g["steps"])]


def assert_same_population(ids, pos, want_ids, want_pos, what):
    """Same agents (any order) at bit-identical positions."""
    assert sorted(ids.tolist()) == sorted(want_ids.tolist()), f"{what}: agent sets differ"
    o, w = np.argsort(ids), np.argsort(want_ids)
    assert np.array_equal(pos[o], want_pos[w]), \
        f"{what}: max deviation {float(np.abs(pos[o] - want_pos[w]).max())} m"


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture
def golden_xml(tmp_path):
    """Writes a golden fixture's scenario to a temporary file; returns (path, fixture)."""
    def _make(name):
        g = load_golden(name)
        p = tmp_path / (name + ".xml")
        p.write_bytes(g["xml"].tobytes())
        return str(p), g
    return _make


def neighbour_lists(g, step):
    off = g[f"nb{step}_off"]
    ids, d2 = g[f"nb{step}_ids"], g[f"nb{step}_d2"]
    return [(ids[off[i]:off[i + 1]], d2[off[i]:off[i + 1]]) for i in range(len(off) - 1)]
