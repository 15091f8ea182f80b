"""Cost-function plugins (the engine's CostFunction plugin API): the example
plugin "ExampleRVO" restates the reference's RVO cost, so a scenario whose
policies name it instead of "RVO" must give the reference's trajectories,
bit for bit, through the plugin dispatch."""
import numpy as np
import pytest

from conftest import load_golden
from umans_gb300 import Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["crossing40_RVO", "obstacle_crossing40_RVO", "toric60_RVO",
                                  "registry40_RandomRVO"])
def test_example_plugin_matches_reference_rvo(name, tmp_path):
    g = load_golden(name)
    xml = g["xml"].tobytes()
    assert b'name="RVO"' in xml
    p = tmp_path / (name + "_plugin.xml")
    p.write_bytes(xml.replace(b'name="RVO"', b'name="ExampleRVO"'))
    sim = Simulation(str(p))
    assert np.array_equal(sim.state()["ids"], g["ids"])
    done = 0
    for k, s in enumerate(g["steps"]):
        if s > 100:
            break
        sim.step(int(s) - done)
        done = int(s)
        pos = sim.positions()
        assert np.array_equal(pos, g["pos"][k]), \
            f"{name} step {s}: max deviation {float(np.abs(pos - g['pos'][k]).max())} m"
