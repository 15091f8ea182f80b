"""Force-based costs (SocialForcesAvoidance, PowerLaw, GoalReachingForce)
under every optimization method run on the force-only kernels: the
four-agents-per-warp kernel in worlds without obstacle edges, the
warp-per-agent one with them.  The velocity then comes from the cost
targets (ForceBasedFunction.cpp:26-52):
- gradient: the gradient step of policy.cpp:78-89;
- global with one cost: its target;
- global with several costs: the default schedule
  (SamplingParameters::ApproximateGlobalOptimization, policy.h:74-86);
- sampling: the first least-cost sample of the policy's schedule
  (costFunction.cpp:60-158).

Trajectories equal the oracle's bit for bit over 60 steps."""
import os

import numpy as np
import pytest

from oracle.port import PortSim
from umans_gb300 import Simulation, scenarios as S

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4

PL_SAMPLING = S.POWERLAW_SAMPLING_POLICY
SF_RANDOM = (
    '<Policy id="{pid}" OptimizationMethod="sampling" SamplingType="random" SamplingBase="current velocity" '
    'SamplingBaseDirection="unit" SamplingAngle="360" RandomSamples="60" SamplingRadius="maximum acceleration" '
    'RelaxationTime="0.5"><costfunction name="SocialForcesAvoidance" range="5"/>'
    '<costfunction name="GoalReachingForce"/></Policy>')
PL_GLOBAL_TWO = (
    '<Policy id="{pid}" OptimizationMethod="global" RelaxationTime="0.5">'
    '<costfunction name="PowerLaw" range="5"/><costfunction name="GoalReachingForce" coeff="2"/></Policy>')
SF_GLOBAL_ONE = (
    '<Policy id="{pid}" OptimizationMethod="global" RelaxationTime="0.5">'
    '<costfunction name="SocialForcesAvoidance" range="5"/></Policy>')
SF_SAMPLING_PREF = (
    '<Policy id="{pid}" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
    'SamplingBaseDirection="preferred velocity" SamplingAngle="180" SpeedSamples="6" AngleSamples="15" '
    'IncludeBaseAsSample="true" SamplingRadius="preferred speed" RelaxationTime="0.3">'
    '<costfunction name="SocialForcesAvoidance" range="4"/><costfunction name="GoalReachingForce"/></Policy>')


def _crossing(policies, n=40, seed=21, pid=None, obstacles=False, toric=False):
    rng = np.random.default_rng(seed)
    h = n // 2
    a = np.stack([rng.uniform(-12, -6, h), rng.uniform(-3, 3, h)], 1)
    b = np.stack([rng.uniform(-3, 3, n - h), rng.uniform(-12, -6, n - h)], 1)
    pos = np.concatenate([a, b])
    goal = np.concatenate([a + [20, 0], b + [0, 20]])
    if pid is None:
        pid = np.zeros(n, np.int64)
    kw = dict(world="Toric", width=30.0, height=30.0) if toric else dict(world="Infinite")
    sc = S.Scenario(dt=0.1, policies=[p.format(pid=k, sfparams="") for k, p in enumerate(policies)],
                    **kw, **S._agents(n, pos, goal, pref=1.3, maxs=1.6, pid=pid))
    if obstacles:
        sc.obstacles = [S.BLOCK.copy()]
    return sc


def _same_as_oracle(path, steps=60, every=5):
    sim = Simulation(path)
    port = PortSim(path, threads=THREADS)
    done = 0
    while done < steps:
        sim.step(every)
        port.step(every)
        done += every
        ref = port.state()["pos"]
        pos = sim.positions()
        assert np.array_equal(pos, ref), f"step {done}: max deviation {float(np.abs(pos - ref).max())} m"
    sim.close()


CASES = {
    "powerlaw_sampling": dict(policies=[PL_SAMPLING]),
    "powerlaw_sampling_obstacle": dict(policies=[PL_SAMPLING], obstacles=True),
    "socialforces_random_sampling_toric": dict(policies=[SF_RANDOM], toric=True),
    "powerlaw_global_two_costs": dict(policies=[PL_GLOBAL_TWO]),
    "socialforces_global_one_cost": dict(policies=[SF_GLOBAL_ONE]),
    "socialforces_sampling_preferred": dict(policies=[SF_SAMPLING_PREF], obstacles=True),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_force_costs_under_each_method_match_oracle(case, tmp_path):
    path = _crossing(**CASES[case]).write(str(tmp_path / f"{case}.xml"))
    _same_as_oracle(path)


def test_mixed_methods_in_one_world_match_oracle(tmp_path):
    """Gradient, sampling and global policies side by side in one kernel group."""
    n = 48
    pid = np.arange(n) % 3
    sc = _crossing([S.SF_POLICY, PL_SAMPLING, PL_GLOBAL_TWO], n=n, seed=22, pid=pid)
    _same_as_oracle(sc.write(str(tmp_path / "mixed.xml")))


def test_batch_powerlaw_sampling_members_match_oracle(tmp_path):
    """PowerLaw-sampling members of the benchmark batch, against the oracle
    (the batch test compares members with their own simulations)."""
    for k in (1, 7, 13):
        n = int(S.batch_counts()[k])
        n = min(n, 400)
        path = S.batch_member(k, n).write(str(tmp_path / f"b{k}.xml"))
        _same_as_oracle(path, steps=30)


@pytest.mark.parametrize("lanes,schedule", [(8, 0), (8, 1), (8, 2), (32, 0), (32, 2)])
def test_launch_shapes_match_oracle(lanes, schedule, tmp_path):
    """Lanes per agent and the agent-to-warp schedule (interleaved,
    contiguous, work list) change no result."""
    n = 48
    pid = np.arange(n) % 2
    path = _crossing([S.SF_POLICY, PL_SAMPLING], n=n, seed=23, pid=pid).write(str(tmp_path / "shape.xml"))
    sim = Simulation(path)
    sim.set_launch(cells_per_range=2.0, warps_per_block=4, occupancy=1.0, schedule=schedule, agent_lanes=lanes)
    port = PortSim(path, threads=THREADS)
    for _ in range(6):
        sim.step(5)
        port.step(5)
        assert np.array_equal(sim.positions(), port.state()["pos"])
    sim.close()


def test_launch_shape_rejects_out_of_range(tmp_path):
    path = _crossing([S.SF_POLICY]).write(str(tmp_path / "bad.xml"))
    sim = Simulation(path)
    for kw in (dict(agent_lanes=16), dict(schedule=3), dict(occupancy=0.0), dict(warps_per_block=0)):
        with pytest.raises(Exception):
            sim.set_launch(**kw)
    sim.step(2)   # still usable
    sim.close()
