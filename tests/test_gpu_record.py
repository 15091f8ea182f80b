"""Trajectory output (the reference's CSVWriter layout at full precision, or
binary chunks): every step's positions, exactly as the simulation had them,
through ring wrap-arounds, agent-list changes and re-run batches."""
import glob
import os

import numpy as np
import pytest

from umans_gb300 import Simulation, read_trajectory, scenarios as S

pytestmark = pytest.mark.gpu


def _stepwise(path, steps):
    s = Simulation(path)
    ids = s.state()["ids"].copy()
    out = []
    for _ in range(steps):
        s.step(1)
        out.append(s.positions().copy())
    s.close()
    return ids, np.array(out)


def _read_csv(d):
    per = {}
    for f in glob.glob(os.path.join(d, "output_*.csv")):
        aid = int(os.path.basename(f)[7:-4])
        rows = [ln.split(",") for ln in open(f).read().splitlines()]
        per[aid] = (np.array([float(r[0]) for r in rows]),
                    np.array([[np.float32(r[1]), np.float32(r[2])] for r in rows], np.float32))
    return per


def test_csv_matches_the_simulation_bit_for_bit(tmp_path):
    path = S.model_crossing("SocialForces").write(str(tmp_path / "x.xml"))
    ids, want = _stepwise(path, 25)
    s = Simulation(path)
    out = str(tmp_path / "csv")
    s.record_start(out, ring_steps=8)
    s.step(10)
    s.step(15)
    s.record_stop()
    per = _read_csv(out)
    assert sorted(per) == sorted(ids.tolist())
    for k, aid in enumerate(ids):
        t, xy = per[int(aid)]
        assert xy.shape == (25, 2)
        assert np.array_equal(xy, want[:, k])               # 9 digits round-trip every float
        assert np.allclose(t, 0.1 * np.arange(1, 26), atol=1e-6)


def test_binary_chunks_and_rerun_batches(tmp_path):
    """Capacity far below the list lengths: batches are restored and re-run;
    the recording holds only the committed steps."""
    path = S.socialforces_toric(n=3000, density=0.625).write(str(tmp_path / "dense.xml"))
    ids, want = _stepwise(path, 12)
    s = Simulation(path, max_neighbours=8)
    out = str(tmp_path / "bin")
    s.record_start(out, ring_steps=5, binary=True)
    s.step(12)
    s.record_stop()
    assert s.max_neighbours > 8
    chunks = read_trajectory(os.path.join(out, "trajectory.bin"))
    assert [c[2].shape[0] for c in chunks] == [5, 5, 2]
    xy = np.concatenate([c[2] for c in chunks])
    assert np.array_equal(chunks[0][0], ids)
    assert np.array_equal(xy, want)


def test_agent_list_changes_flush_the_ring(tmp_path):
    path = S.model_crossing("PowerLaw", n=30).write(str(tmp_path / "p.xml"))
    s = Simulation(path)
    out = str(tmp_path / "dyn")
    s.record_start(out, ring_steps=64)
    s.step(4)
    new_id = s.add_agent(5.0, 5.0, 0.3, 1.3, 1.6, 5.0, 0)
    s.step(3)
    s.remove_agent(0)
    s.step(2)
    final = dict(zip(s.state()["ids"].tolist(), s.positions()))
    s.record_stop()
    per = _read_csv(out)
    assert len(per[new_id][0]) == 5          # steps 5..9
    assert len(per[0][0]) == 7               # steps 1..7, then removed
    assert len(per[1][0]) == 9
    for aid, p in final.items():
        assert np.array_equal(per[aid][1][-1], p)


def test_batch_records_each_scenario_as_its_own_simulation(tmp_path):
    """A batch writes scenario k into <dir>/scenario_k, the same files its own
    simulation writes: binary chunks through ring wrap-arounds, and CSV
    with a member whose agents arrive and leave (the list changes flush the
    ring) and a member with another time step."""
    from conftest import load_golden
    from umans_gb300 import Batch
    arr = load_golden("arrivals40_SocialForces")
    p_arr = tmp_path / "arrivals.xml"
    p_arr.write_bytes(arr["xml"].tobytes())
    slow = S.model_crossing("PowerLaw", n=24)
    slow.dt = 0.05
    paths = [S.model_crossing("SocialForces", n=30).write(str(tmp_path / "a.xml")), str(p_arr),
             slow.write(str(tmp_path / "c.xml"))]
    for fmt in (True, False):
        out = str(tmp_path / ("bbin" if fmt else "bcsv"))
        b = Batch(paths)
        b.record_start(out, ring_steps=7, binary=fmt)
        b.step(9)
        b.step(8)
        b.record_stop()
        b.close()
        for k, p in enumerate(paths):
            own = str(tmp_path / f"own{k}_{fmt}")
            s = Simulation(p)
            s.record_start(own, ring_steps=64, binary=fmt)
            s.step(17)
            s.record_stop()
            s.close()
            got_dir = os.path.join(out, f"scenario_{k}")
            if fmt:
                got = _per_agent(read_trajectory(os.path.join(got_dir, "trajectory.bin")))
                want = _per_agent(read_trajectory(os.path.join(own, "trajectory.bin")))
            else:
                got, want = _read_csv(got_dir), _read_csv(own)
            assert sorted(got) == sorted(want), f"scenario {k}"
            for aid in want:
                assert np.array_equal(got[aid][1], want[aid][1]), f"scenario {k} agent {aid}"
                assert np.array_equal(got[aid][0], want[aid][0])


def _per_agent(chunks):
    """Binary chunks as {id: (times, xy)} (agents may join or leave between chunks)."""
    per = {}
    for ids, times, xy in chunks:
        for j, aid in enumerate(ids.tolist()):
            t, p = per.get(aid, ([], []))
            per[aid] = (t + list(times), p + [xy[:, j]])
    return {a: (np.array(t), np.concatenate(p)) for a, (t, p) in per.items()}
