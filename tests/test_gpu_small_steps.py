"""Small worlds with the steps of one call in one launch (k_small_steps: a
block that builds the grid and updates the agents step after step) against
the oracle and against the one-graph-launch-per-step path, bit for bit.

The reference steps its world one DoStep at a time (worldBase.cpp:79-128,
crowdSimulator.cpp:77-95); running several steps inside one launch changes
no result."""
import os

import numpy as np
import pytest

from oracle.port import PortSim
from umans_gb300 import Simulation, scenarios as S

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def _run(path, calls, multi=True):
    sim = Simulation(path)
    sim.set_multi_step(multi)
    out = []
    for k in calls:
        sim.step(k)
        out.append(sim.positions())
    t = sim.time
    sim.close()
    return out, t


def _oracle(path, calls):
    port = PortSim(path, threads=THREADS)
    out = []
    for k in calls:
        port.step(k)
        out.append(port.state()["pos"])
    return out


def _check(path, calls):
    got, t1 = _run(path, calls, True)
    per_step, t0 = _run(path, calls, False)
    ref = _oracle(path, calls)
    done = 0
    for k, g, p, r in zip(calls, got, per_step, ref):
        done += k
        assert np.array_equal(g, p), f"after {done} steps: one launch differs from one launch per step"
        assert np.array_equal(g, r), f"after {done} steps: max deviation {float(np.abs(g - r).max())} m"
    assert t1 == t0


def test_orca_circle_300_steps_in_one_call(tmp_path):
    """The small ORCA circle (50 agents, 300 steps) run by one call."""
    path = S.circle_orca().write(str(tmp_path / "circle.xml"))
    _check(path, [300])


@pytest.mark.parametrize("model", ["ORCA", "RVO", "Karamouzas", "Moussaid", "Paris", "Dutra"])
def test_models_several_steps_per_call(model, tmp_path):
    """The general (RVO, Moussaid, Paris, Dutra), ORCA and Karamouzas
    kernels, calls of 1, 7 and 32 steps."""
    path = S.model_circle(model).write(str(tmp_path / f"{model}.xml"))
    _check(path, [1, 7, 32])


@pytest.mark.parametrize("model", ["ORCA", "RVO"])
def test_obstacles_and_toric_worlds(model, tmp_path):
    _check(S.model_obstacle_crossing(model).write(str(tmp_path / "obst.xml")), [25, 15])
    _check(S.model_toric(model).write(str(tmp_path / "toric.xml")), [25, 15])


@pytest.mark.parametrize("model", ["ORCA", "Moussaid"])
def test_thousand_agents_eight_warps_per_block(model, tmp_path):
    """Above 512 agents the launch takes blocks of 8 warps."""
    path = S.model_toric(model, n=1024, side=60.0).write(str(tmp_path / "k.xml"))
    _check(path, [12, 8])


def test_neighbour_capacity_grows_inside_one_call(tmp_path):
    """200 agents converging on the circle's centre: the neighbour lists
    outgrow the capacity chosen from the initial state during the call, the
    host re-runs the call's steps from its snapshot with a larger capacity,
    and the trajectory is the oracle's."""
    path = S.model_circle("ORCA", n=200, radius_m=25.0).write(str(tmp_path / "dense.xml"))
    sim = Simulation(path)
    cap0 = sim.max_neighbours
    sim.close()
    _check(path, [300])
    sim = Simulation(path)
    sim.step(300)
    assert sim.max_neighbours > cap0
    sim.close()


def test_dynamic_population_and_recording_take_the_per_step_path(tmp_path):
    """Worlds that need host work between steps (agents joining and leaving,
    trajectory output) step one launch at a time, with the same results."""
    path = S.model_arrivals("ORCA").write(str(tmp_path / "arrivals.xml"))
    _check(path, [20, 40])
    sim = Simulation(S.circle_orca().write(str(tmp_path / "rec.xml")))
    sim.record_start(str(tmp_path / "out"), ring_steps=16)
    sim.step(40)
    sim.record_stop()
    pos = sim.positions()
    sim.close()
    ref = _oracle(str(tmp_path / "rec.xml"), [40])[0]
    assert np.array_equal(pos, ref)
