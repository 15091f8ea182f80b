"""Cost-function plugins (the engine's CostFunction plugin API), through the
plugin dispatch, bit for bit:

* "ExampleRVO" restates the reference's RVO cost (GetCost only): scenarios
  naming it instead of "RVO" give the reference's trajectories;
* "ExampleFOE" restates FOEAvoidance with its closed-form GetGradient
  override: the gradient-method FOEAvoidance fixtures (which the default
  finite-difference gradient would not reproduce);
* "ExampleGoal" restates GoalReachingForce with GetGradient and
  GetGlobalMinimum overrides: the same trajectories as GoalReachingForce,
  under the global method (its closed form instead of the default
  sampling) and the gradient method, and the oracle's."""
import numpy as np
import pytest

from conftest import load_golden
from oracle.port import PortSim
from umans_gb300 import Simulation, scenarios as S

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


def _run_fixture_renamed(name, old, new, tmp_path):
    g = load_golden(name)
    xml = g["xml"].tobytes()
    assert old in xml
    p = tmp_path / (name + "_plugin.xml")
    p.write_bytes(xml.replace(old, new))
    sim = Simulation(str(p))
    done = 0
    for k, s in enumerate(g["steps"]):
        if s > 100:
            break
        sim.step(int(s) - done)
        done = int(s)
        pos = sim.positions()
        assert np.array_equal(pos, g["pos"][k]), \
            f"{name} step {s}: max deviation {float(np.abs(pos - g['pos'][k]).max())} m"


@pytest.mark.parametrize("name", ["crossing40_FOEAvoidance", "obstacle_crossing40_FOEAvoidance",
                                  "toric60_FOEAvoidance"])
def test_plugin_gradient_override_matches_reference_foe(name, tmp_path):
    _run_fixture_renamed(name, b'name="FOEAvoidance"', b'name="ExampleFOE"', tmp_path)


@pytest.mark.parametrize("method", ["global", "gradient"])
def test_plugin_global_minimum_and_gradient_overrides(method, tmp_path):
    rng = np.random.default_rng(11)
    n = 40
    pos = rng.uniform(-8, 8, (n, 2))
    goal = -pos + rng.uniform(-1, 1, (n, 2))
    final = {}
    for cost in ("GoalReachingForce", "ExampleGoal"):
        pol = (f'<Policy id="0" OptimizationMethod="{method}" RelaxationTime="0.5">'
               f'<costfunction name="{cost}" agentMass="1.5"/></Policy>')
        path = S.Scenario(dt=0.1, world="Infinite", policies=[pol], **S._agents(n, pos, goal)).write(
            str(tmp_path / f"{method}_{cost}.xml"))
        sim = Simulation(path)
        sim.step(60)
        final[cost] = sim.positions()
        if cost == "GoalReachingForce":
            port = PortSim(path)
            port.step(60)
            assert np.array_equal(final[cost], port.state()["pos"])
    assert np.array_equal(final["GoalReachingForce"], final["ExampleGoal"])
