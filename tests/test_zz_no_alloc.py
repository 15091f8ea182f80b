"""The allocation-free ORCA entry point (umans_orca_velocities_noalloc).

It exists for callers that cannot allocate GPU memory when they need a
result (an application that owns all device memory through its own pool and
forbids cudaMalloc after start-up).  Its ORCA line buffers are a static
device array shared by all calls.  These tests call it through the C ABI:
two calls in a row (the first on the null stream, the second on a stream of
their own) must give exactly the velocities of the regular engine step for
the same state (the engine uses allocated per-warp scratch, and both run the
same line construction and linear programs, so the tolerance is zero); a
count above the capacity and an index outside the agents are reported with
UMANS_ERR_DEVICE; n = 0 does nothing.  The file is collected last so that a
failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from umans_gb300 import Simulation, _lib, scenarios as S

pytestmark = pytest.mark.gpu
TOL = 0.0   # bit-identical to the engine's step

POLICY = ('<Policy id="0" OptimizationMethod="global" RelaxationTime="0" ContactForceScale="0">'
          '<costfunction name="ORCA" range="5" timeHorizon="5"/></Policy>')
UMANS_ERR_DEVICE = 4


def _scenario(tmp_path, n=3000):
    rng = np.random.default_rng(21)
    side = float(np.sqrt(n / 0.5))
    pos = rng.uniform(-side / 2, side / 2, (n, 2))
    goal = rng.uniform(-side / 2, side / 2, (n, 2))
    sc = S.Scenario(dt=0.1, world="Infinite", policies=[POLICY], **S._agents(n, pos, goal))
    return sc.write(str(tmp_path / "orca_noalloc.xml"))


def _call(lib, torch, n, arrays, cap, out, stream=None):
    p = lambda t: C.c_void_p(t.data_ptr())
    a = arrays
    return lib.umans_orca_velocities_noalloc(n, p(a["pos"]), p(a["vel"]), p(a["pref"]), p(a["radius"]),
                                             p(a["max_speed"]), p(a["max_accel"]), p(a["nbr"]), p(a["nd2"]),
                                             p(a["ncnt"]), cap, 5.0, 5.0, 0.1, 0.0, p(out), stream)


def _arrays(torch, n, state, prefvel, ids, d2, cnt):
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    return dict(pos=dev(state["pos"]), vel=dev(state["vel"]), pref=dev(prefvel),
                radius=dev(np.full(n, 0.3, np.float32)), max_speed=dev(np.full(n, 1.8, np.float32)),
                max_accel=dev(np.full(n, 5.0, np.float32)), nbr=dev(ids.astype(np.int32)),
                nd2=dev(d2.astype(np.float32)), ncnt=dev(cnt.astype(np.int32)))


def test_noalloc_matches_engine_step_twice(tmp_path):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    sim = Simulation(_scenario(tmp_path))
    sim.step(5)
    n = sim.n
    side = torch.cuda.Stream()
    for call in range(2):
        before = sim.state()
        ids, d2, cnt = sim.neighbours(cap=128)
        assert np.array_equal(before["ids"], np.arange(n))   # ids are list slots here
        sim.step(1)
        after = sim.state()   # velocity chosen by the engine, preferred velocity it used
        arrays = _arrays(torch, n, before, after["prefvel"], ids, d2, cnt)
        out = torch.full((n, 2), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        stream = None if call == 0 else C.c_void_p(side.cuda_stream)
        rc = _call(lib, torch, n, arrays, 128, out, stream)
        assert rc == 0, lib.umans_last_error(None)
        got = out.cpu().numpy()
        dev_max = float(np.abs(got - after["vel"]).max())
        print(f"call {call}: max |v_noalloc - v_engine| = {dev_max:.3g} m/s")
        assert dev_max <= TOL
    sim.close()


def test_noalloc_reports_truncated_lists(tmp_path):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    sim = Simulation(_scenario(tmp_path, n=500))
    n = sim.n
    ids, d2, cnt = sim.neighbours(cap=8)
    assert int(cnt.max()) > 8   # some lists are longer than the capacity given below
    st = sim.state()
    arrays = _arrays(torch, n, st, st["prefvel"], ids, d2, cnt)
    out = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = _call(lib, torch, n, arrays, 8, out)
    assert rc == UMANS_ERR_DEVICE
    assert b"exceeds nbr_cap" in lib.umans_last_error(None)
    assert np.isfinite(out.cpu().numpy()).all()
    sim.close()


def test_noalloc_skips_index_outside_agents():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    n, cap = 4, 2
    pos = np.array([[0, 0], [1, 0], [0, 1], [3, 3]], np.float32)
    st = dict(pos=pos, vel=np.zeros((n, 2), np.float32))
    pref = np.array([[1, 0], [-1, 0], [0, -1], [0, 1]], np.float32)
    ids = np.array([[1, n], [0, 2], [0, 1], [0, 0]], np.int32)   # agent 0 lists index n
    d2 = np.array([[1, 1], [1, 2], [1, 2], [0, 0]], np.float32)
    cnt = np.array([2, 2, 2, 0], np.int32)
    arrays = _arrays(torch, n, st, pref, ids, d2, cnt)
    out = torch.full((n, 2), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = _call(lib, torch, n, arrays, cap, out)
    assert rc == UMANS_ERR_DEVICE
    assert b"outside [0, n)" in lib.umans_last_error(None)
    assert np.isfinite(out.cpu().numpy()).all()   # every agent still gets a velocity


def test_noalloc_zero_agents():
    lib = _lib.load()
    rc = lib.umans_orca_velocities_noalloc(0, None, None, None, None, None, None, None, None, None, 128,
                                           5.0, 5.0, 0.1, 0.0, None, None)
    assert rc == 0


def test_noalloc_rejects_oversized_lists():
    lib = _lib.load()
    rc = lib.umans_orca_velocities_noalloc(1, None, None, None, None, None, None, None, None, None, 129,
                                           5.0, 5.0, 0.1, 0.0, None, None)
    assert rc == 1
    assert b"exceeds the 128 ORCA lines" in lib.umans_last_error(None)
