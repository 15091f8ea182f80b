"""The reference-compatible C functions and the handle API (GPU)."""
import numpy as np
import pytest

from oracle.port import PortSim
from umans_gb300 import UMANS, AgentData, Simulation, UmansError, scenarios as S

pytestmark = pytest.mark.gpu


def test_reference_api_roundtrip(tmp_path):
    path = S.model_crossing("SocialForces").write(str(tmp_path / "x.xml"))
    u = UMANS()
    assert u.doSimulationSteps(1) is False        # no simulation yet
    assert u.startSimulation(path, 4)
    assert abs(u.getSimulationTimeStep() - 0.1) < 1e-7
    assert u.doSimulationSteps(10)
    agents = u.getAgentPositions()
    assert len(agents) == 40 and agents[0].id == 0
    port = PortSim(path)
    port.step(10)
    pos = np.array([[a.position_x, a.position_y] for a in agents], np.float32)
    assert np.abs(pos - port.state()["pos"]).max() <= 1e-4
    # SetAgentPositions by id, unknown ids skipped
    moved = [AgentData(3, 1.0, 2.0, 0.5, 0.0, 1.0, 0.0), AgentData(999, 0, 0, 0, 0, 1, 0)]
    assert u.setAgentPositions(moved)
    a3 = [a for a in u.getAgentPositions() if a.id == 3][0]
    assert (a3.position_x, a3.position_y, a3.velocity_x) == (1.0, 2.0, 0.5)
    new_id = u.addAgent(5.0, 5.0, 0.3, 1.3, 1.6, 5.0, 0, -1)
    assert new_id == 40
    assert u.setAgentGoal(new_id, 6.0, 5.0)
    assert u.removeAgent(0)
    assert not u.removeAgent(12345)
    ids = [a.id for a in u.getAgentPositions()]
    assert 0 not in ids and ids[0] == 40      # the last agent moved into the gap
    assert u.doSimulationSteps(5)
    assert u.cleanUp()
    assert not u.cleanUp()


def test_bad_scenarios_fail_loudly(tmp_path):
    p = tmp_path / "bad.xml"
    p.write_text('<Simulation delta_time="0.1"><World type="Infinite"/><Policies>'
                 '<Policy id="0" OptimizationMethod="global"><costfunction name="ORCA"/>'
                 '<costfunction name="ORCA"/></Policy></Policies></Simulation>')
    with pytest.raises(UmansError, match="not supported"):
        Simulation(str(p))
    p.write_text('<Simulation delta_time="0.1"><World type="Infinite"/><Policies>'
                 '<Policy id="0" OptimizationMethod="gradient"><costfunction name="NoSuchCost"/>'
                 '</Policy></Policies></Simulation>')
    with pytest.raises(UmansError, match="cost function"):
        Simulation(str(p))
    p.write_text('<Simulation delta_time="-1"><World type="Infinite"/></Simulation>')
    with pytest.raises(UmansError, match="delta_time"):
        Simulation(str(p))
    with pytest.raises(UmansError):
        Simulation(str(tmp_path / "missing.xml"))


def test_empty_world_and_single_agent(tmp_path):
    p = tmp_path / "e.xml"
    p.write_text('<Simulation delta_time="0.1"><World type="Toric" width="10" height="10"/><Policies>'
                 '<Policy id="0" OptimizationMethod="gradient"><costfunction name="GoalReachingForce"/>'
                 '</Policy></Policies></Simulation>')
    s = Simulation(str(p))
    s.step(3)
    assert s.n == 0
    i = s.add_agent(0, 0, 0.3, 1.3, 1.8, 5.0, 0)
    s.set_goal(i, 3, 0)
    s.step(5)
    assert s.positions()[0, 0] > 0.1


def test_returned_buffer_fed_back_and_pageable_input(tmp_path):
    """The e2e loop: the (page-locked) buffer GetAgentPositions returns is sent
    back by SetAgentPositions; a pageable copy gives the same result."""
    import ctypes as C
    from umans_gb300 import _lib
    path = S.model_crossing("SocialForces", n=60).write(str(tmp_path / "x.xml"))
    lib = _lib.load()
    ref = Simulation(path)
    ref.step(8)
    want = ref.state()
    assert lib.StartSimulation(path.encode(), 1)
    ptr = C.POINTER(AgentData)()
    n = C.c_int()
    cur = None
    for k in range(8):
        if cur is not None:
            assert lib.SetAgentPositions(cur, n.value)
        assert lib.DoSimulationSteps(1)
        assert lib.GetAgentPositions(C.byref(ptr), C.byref(n))
        cur = ptr if k % 2 == 0 else (AgentData * n.value).from_buffer_copy(
            C.string_at(ptr, C.sizeof(AgentData) * n.value))
    pos = np.array([[ptr[i].position_x, ptr[i].position_y] for i in range(n.value)], np.float32)
    vel = np.array([[ptr[i].velocity_x, ptr[i].velocity_y] for i in range(n.value)], np.float32)
    assert np.array_equal(pos, want["pos"]) and np.array_equal(vel, want["vel"])
    assert lib.CleanUp()


def test_async_steps_then_host_reads(tmp_path):
    path = S.model_crossing("PowerLaw", n=50).write(str(tmp_path / "p.xml"))
    a, b = Simulation(path), Simulation(path)
    for _ in range(5):
        a.step_async(2)
    b.step(10)
    assert np.array_equal(a.positions(), b.positions())
    assert a.time == b.time
