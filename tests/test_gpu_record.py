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
