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


def golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


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
