"""The batched form: many independent scenarios stepped together must give
each scenario exactly the trajectory it has on its own (and, through the
golden fixtures, the reference's)."""
import numpy as np
import pytest

from conftest import assert_same_population, dynamic_golden_names, dynamic_snapshots, golden_names, load_golden
from umans_gb300 import Batch, Simulation, scenarios as S

pytestmark = pytest.mark.gpu


def _mixed(tmp_path, count=24, cap=300):
    counts = np.minimum(S.batch_counts(num=count, seed=4), cap)
    return [S.batch_member(k, int(n)).write(str(tmp_path / f"m{k}.xml")) for k, n in enumerate(counts)]


def test_batch_equals_individual_simulations(tmp_path):
    paths = _mixed(tmp_path)
    b = Batch(paths)
    off = b.offsets
    assert off[0] == 0 and len(off) == len(paths) + 1
    b.step(25)
    pos = b.positions()
    for k, p in enumerate(paths):
        s = Simulation(p)
        s.step(25)
        assert np.array_equal(pos[off[k]:off[k + 1]], s.positions()), f"scenario {k}"


def test_full_batch_members_equal_their_simulations(tmp_path):
    """The benchmark's batch of 4096 scenarios (agent counts log-uniform in
    [8, 2048], ~1.5M agents) stepped 20 steps together: 64 members (every
    64th, all three policy kinds and both layouts) equal their own
    simulations exactly."""
    counts = S.batch_counts()
    assert len(counts) == 4096
    paths = [S.batch_member(k, int(n)).write(str(tmp_path / f"b{k}.xml")) for k, n in enumerate(counts)]
    b = Batch(paths)
    off = b.offsets
    b.step(20)
    pos = b.positions()
    b.close()
    sample = list(range(0, 4096, 64))
    kinds = {k % 3 for k in sample}
    assert kinds == {0, 1, 2}
    worst = 0.0
    for k in sample:
        s = Simulation(paths[k])
        s.step(20)
        d = float(np.abs(pos[off[k]:off[k + 1]] - s.positions()).max())
        worst = max(worst, d)
        s.close()
        assert d == 0.0, f"scenario {k} ({int(counts[k])} agents): {d} m"
    print(f"4096-scenario batch, 20 steps: {len(sample)} members, max deviation {worst:.3g} m")


def test_autotune_keeps_results(tmp_path):
    paths = _mixed(tmp_path, count=12)
    a, b = Batch(paths), Batch(paths)
    a.step(3)
    b.step(3)
    choice = b.autotune(trial_steps=2)
    assert choice["cells_per_range"] > 0 and choice["warps_per_block"] in (2, 4)
    assert choice["agent_lanes"] in (8, 32)
    a.step(10)
    b.step(10)
    assert np.array_equal(a.positions(), b.positions())


def test_batch_with_dynamic_population_matches_reference(tmp_path):
    """Timed insertion and removal at the goal (worldBase.cpp:82-86, 122-127)
    in a batch.  The eleven arrivals fixtures are interleaved with static
    members.  At every snapshot each member holds the fixture's agents at
    bit-identical positions, and the static members equal their own
    simulations."""
    names = dynamic_golden_names()
    fixtures = [load_golden(n) for n in names]
    paths, members = [], []
    for k, (name, g) in enumerate(zip(names, fixtures)):
        p = tmp_path / (name + ".xml")
        p.write_bytes(g["xml"].tobytes())
        paths.append(str(p))
        members.append(("fixture", g, name))
        if k % 3 == 0:
            q = S.batch_member(k, 30).write(str(tmp_path / f"static{k}.xml"))
            paths.append(q)
            members.append(("static", Simulation(q), q))
    b = Batch(paths)
    snaps = [dict((s, (ids, pos)) for s, ids, pos in dynamic_snapshots(g)) if kind == "fixture" else None
             for kind, g, _ in members]
    steps = sorted({s for d in snaps if d for s in d})
    done = 0
    for s in steps:
        b.step(s - done)
        for kind, obj, _ in members:
            if kind == "static":
                obj.step(s - done)
        done = s
        off = b.offsets
        st = b.state()
        for m, (kind, obj, what) in enumerate(members):
            ids, pos = st["ids"][off[m]:off[m + 1]], st["pos"][off[m]:off[m + 1]]
            if kind == "fixture":
                if s in snaps[m]:
                    want_ids, want_pos = snaps[m][s]
                    assert_same_population(ids, pos, want_ids, want_pos, f"{what} step {s}")
            else:
                ref = obj.state()
                assert np.array_equal(ids, ref["ids"]) and np.array_equal(pos, ref["pos"]), f"{what} step {s}"


def test_work_list_schedule_keeps_results(tmp_path):
    """The work-list schedule (warps taking agent tiles from a counter) and
    32 lanes per agent give the batch the same trajectories."""
    paths = _mixed(tmp_path, count=12)
    a, b = Batch(paths), Batch(paths)
    b.set_launch(schedule=2, agent_lanes=32)
    for _ in range(3):
        a.step(4)
        b.step(4)
        assert np.array_equal(a.positions(), b.positions())
    b.set_launch(schedule=2, agent_lanes=8)
    a.step(4)
    b.step(4)
    assert np.array_equal(a.positions(), b.positions())


def test_batch_of_golden_scenarios_matches_reference(golden_xml):
    names = golden_names()
    items = [golden_xml(n) for n in names]
    b = Batch([p for p, _ in items])
    off = b.offsets
    snaps = sorted({int(s) for _, g in items for s in g["steps"] if s <= 100})
    done = 0
    for s in snaps:
        b.step(s - done)
        done = s
        pos = b.positions()
        for k, (name, (_, g)) in enumerate(zip(names, items)):
            idx = np.nonzero(g["steps"] == s)[0]
            if len(idx):
                dev = float(np.abs(pos[off[k]:off[k + 1]] - g["pos"][idx[0]]).max()) if off[k + 1] > off[k] else 0.0
                assert dev == 0.0, f"{name} step {s}: {dev}"


def test_batch_with_obstacles_equals_individual_simulations(tmp_path):
    """Scenarios with static obstacles (each its own edges) in one batch."""
    scs = [S.model_obstacle_crossing("SocialForces"), S.model_corridor_walls("Karamouzas"),
           S.model_toric_obstacle("ORCA"), S.model_crossing("PowerLaw")]
    paths = [sc.write(str(tmp_path / f"o{k}.xml")) for k, sc in enumerate(scs)]
    b = Batch(paths)
    off = b.offsets
    b.step(30)
    pos = b.positions()
    for k, p in enumerate(paths):
        s = Simulation(p)
        s.step(30)
        assert np.array_equal(pos[off[k]:off[k + 1]], s.positions()), f"scenario {k}"
