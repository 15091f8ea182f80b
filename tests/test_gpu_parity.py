"""Parity of the CUDA engine with the reference, through the C ABI.

* trajectories against the golden fixtures made by the reference engine:
  max per-agent position deviation <= 1e-4 m over the first 100 steps;
* neighbour lists against the reference's lists (same ids, same order up to
  distance ties) and, on arbitrary positions, against the CPU oracle;
* the benchmark workloads at full size against the CPU oracle (the
  100k-agent toric SocialForces crowd over its first 100 steps, the
  Karamouzas corridor at 100k agents over 20 steps), plus size-independent
  properties (determinism, finiteness, no capacity overflow).
"""
import os

import numpy as np
import pytest

from conftest import assert_same_population, dynamic_golden_names, dynamic_snapshots, golden_names, neighbour_lists
from oracle.port import PortSim
from test_oracle_golden import assert_same_list
from umans_gb300 import Simulation, scenarios as S

pytestmark = pytest.mark.gpu
TOL = 1e-4   # m over the first 100 steps (the parity bound)
THREADS = os.cpu_count() or 4


# every fixture is asserted over its first 100 steps (the host sinf/cosf of
# the TtcaDca and FOEAvoidance gradient rotations, the random-sample rotations
# and the segment collision times are reproduced exactly on the device)
BOUNDED_STEPS = {}


@pytest.mark.parametrize("name", golden_names())
def test_trajectory_matches_reference(name, golden_xml):
    path, g = golden_xml(name)
    horizon = next((v for k, v in BOUNDED_STEPS.items() if name.endswith("_" + k)), 100)
    sim = Simulation(path)
    assert np.array_equal(sim.state()["ids"], g["ids"])
    done, worst, worst_all = 0, 0.0, 0.0
    for k, s in enumerate(g["steps"]):
        sim.step(int(s) - done)
        done = int(s)
        pos = sim.positions()
        dev = float(np.abs(pos - g["pos"][k]).max()) if len(pos) else 0.0
        assert np.isfinite(pos).all()
        if s <= horizon:
            worst = max(worst, dev)
        if s <= 100:
            worst_all = max(worst_all, dev)
    print(f"{name}: max deviation over the first {min(done, horizon)} steps = {worst:.3g} m; "
          f"over {min(done, 100)} steps = {worst_all:.3g} m")
    assert worst <= TOL, f"{name}: max deviation {worst} m"
    assert worst_all == 0.0, f"{name}: not bit-identical ({worst_all} m)"


@pytest.mark.parametrize("name", dynamic_golden_names())
def test_dynamic_population_matches_reference(name, golden_xml):
    """Timed insertion and remove-at-goal (worldBase.cpp:79-86, 124-127): the
    same agents at bit-identical positions at every snapshot."""
    path, g = golden_xml(name)
    sim = Simulation(path)
    done = 0
    for s, ids, pos in dynamic_snapshots(g):
        sim.step(s - done)
        done = s
        st = sim.state()
        assert_same_population(st["ids"], st["pos"], ids, pos, f"{name} step {s}")


@pytest.mark.parametrize("name", [n for n in golden_names() if n.startswith(("toric60", "orca_circle50",
                                                                          "socialforces_toric", "karamouzas"))])
def test_neighbour_lists_match_reference(name, golden_xml):
    path, g = golden_xml(name)
    sim = Simulation(path)
    ref = neighbour_lists(g, 1)
    ids, d2, cnt = sim.neighbours(cap=512)
    for i, (rid, rd2) in enumerate(ref):
        k = int(cnt[i])
        assert_same_list(ids[i, :k], d2[i, :k], rid, rd2, f"{name} agent {i}")


@pytest.mark.parametrize("world", ["toric", "infinite"])
def test_neighbour_lists_match_oracle_on_random_states(world, tmp_path):
    rng = np.random.default_rng(7)
    if world == "toric":
        sc = S.socialforces_toric(n=4000, density=0.625)
    else:
        sc = S.karamouzas_corridor(n=3000, width=30.0)
    path = sc.write(str(tmp_path / "s.xml"))
    sim = Simulation(path)
    port = PortSim(path, threads=THREADS)
    for trial in range(3):
        pos = sim.positions() + rng.normal(0, 0.5, (sim.n, 2)).astype(np.float32)
        if world == "toric":
            h = sc.width / 2
            pos = np.clip(pos, -h, h).astype(np.float32)
        sim.set_state(pos=pos)
        port.set_state(pos=pos)
        ids, d2, cnt = sim.neighbours(cap=1024)
        port.step(1)   # builds the port's lists from `pos`
        pids = port.state()["ids"]
        for i in range(sim.n):
            rid, rd2, _ = port.neighbors(i)
            k = int(cnt[i])
            assert_same_list(ids[i, :k], d2[i, :k], rid.astype(np.int32), rd2, f"trial {trial} agent {pids[i]}")


def _compare_with_port(path, steps, every=1):
    """Max per-agent position deviation from the oracle, compared every
    `every` steps and after the last."""
    sim = Simulation(path)
    port = PortSim(path, threads=THREADS)
    worst, done = 0.0, 0
    while done < steps:
        k = min(every, steps - done)
        sim.step(k)
        port.step(k)
        done += k
        worst = max(worst, float(np.abs(sim.positions() - port.state()["pos"]).max()))
    return worst


def test_full_size_socialforces_matches_oracle(tmp_path):
    """The plain large workload (100k agents, 400 x 400 m toric world) over
    its first 100 steps, the horizon of the 1e-4 m bar."""
    path = S.socialforces_toric().write(str(tmp_path / "sf100k.xml"))
    worst = _compare_with_port(path, 100, every=5)
    print(f"100k SocialForces toric: max deviation over 100 steps = {worst:.3g} m")
    assert worst <= TOL


def test_karamouzas_corridor_matches_oracle(tmp_path):
    """The sampling-heavy corridor at 100k agents (1000 x 100 m, the full
    workload's density and width) over 20 steps."""
    path = S.karamouzas_corridor(n=100_000, width=100.0).write(str(tmp_path / "k100k.xml"))
    worst = _compare_with_port(path, 20, every=5)
    print(f"100k Karamouzas corridor: max deviation over 20 steps = {worst:.3g} m")
    assert worst <= TOL


def test_full_size_properties(tmp_path):
    """100k agents: deterministic, finite, no neighbour-capacity overflow."""
    path = S.socialforces_toric().write(str(tmp_path / "sf100k.xml"))
    a, b = Simulation(path), Simulation(path)
    a.step(20)
    b.step(20)
    pa, pb = a.positions(), b.positions()
    assert np.array_equal(pa, pb)
    assert np.isfinite(pa).all()
    assert np.abs(pa).max() <= 200.0 + 1e-3   # toric wrap keeps agents in the box


def test_capacity_overflow_reruns_batch_exactly(tmp_path):
    """A neighbour capacity far below the list lengths: every overflowing
    batch is restored from its snapshot and re-run with a doubled capacity,
    so the trajectory still equals the oracle's."""
    path = S.socialforces_toric(n=3000, density=0.625).write(str(tmp_path / "dense.xml"))
    sim = Simulation(path, max_neighbours=8)
    port = PortSim(path, threads=THREADS)
    sim.step(15)
    port.step(15)
    assert sim.max_neighbours > 8
    assert np.array_equal(sim.positions(), port.state()["pos"])
