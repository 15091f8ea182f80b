"""The allocation-free ORCA entry point (umans_orca_velocities_noalloc).

It exists for callers that cannot allocate GPU memory when they need a
result (an application that owns all device memory through its own pool and
forbids cudaMalloc after start-up).  Its ORCA line buffers are a static
device array shared by all calls.  This file checks, through the C ABI, that
two calls in a row give the velocities the regular engine step computes for
the same state (the engine's step uses allocated per-warp scratch), within
the tolerance the parity tests use.  It is collected last so that a failure
here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from umans_gb300 import Simulation, _lib, scenarios as S

pytestmark = pytest.mark.gpu
TOL = 1e-4

POLICY = ('<Policy id="0" OptimizationMethod="global" RelaxationTime="0" ContactForceScale="0">'
          '<costfunction name="ORCA" range="5" timeHorizon="5"/></Policy>')


def _scenario(tmp_path, n=3000):
    rng = np.random.default_rng(21)
    side = float(np.sqrt(n / 0.5))
    pos = rng.uniform(-side / 2, side / 2, (n, 2))
    goal = rng.uniform(-side / 2, side / 2, (n, 2))
    sc = S.Scenario(dt=0.1, world="Infinite", policies=[POLICY], **S._agents(n, pos, goal))
    return sc.write(str(tmp_path / "orca_noalloc.xml"))


def test_noalloc_matches_engine_step_twice(tmp_path):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    sim = Simulation(_scenario(tmp_path))
    sim.step(5)
    n = sim.n
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    radius = dev(np.full(n, 0.3, np.float32))
    max_speed = dev(np.full(n, 1.8, np.float32))
    max_accel = dev(np.full(n, 5.0, np.float32))
    for call in range(2):
        before = sim.state()
        ids, d2, cnt = sim.neighbours(cap=128)
        assert np.array_equal(before["ids"], np.arange(n))   # ids are list slots here
        sim.step(1)
        after = sim.state()   # velocity chosen by the engine, preferred velocity it used
        pos, vel, pref = dev(before["pos"]), dev(before["vel"]), dev(after["prefvel"])
        nbr, nd2, ncnt = dev(ids), dev(d2), dev(cnt)
        out = torch.full((n, 2), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        p = lambda t: C.c_void_p(t.data_ptr())
        rc = lib.umans_orca_velocities_noalloc(n, p(pos), p(vel), p(pref), p(radius), p(max_speed), p(max_accel),
                                               p(nbr), p(nd2), p(ncnt), 128, 5.0, 5.0, 0.1, 0.0, p(out), None)
        assert rc == 0, lib.umans_last_error(None)
        got = out.cpu().numpy()
        dev_max = float(np.abs(got - after["vel"]).max())
        print(f"call {call}: max |v_noalloc - v_engine| = {dev_max:.3g} m/s")
        assert dev_max <= TOL


def test_noalloc_rejects_oversized_lists():
    lib = _lib.load()
    rc = lib.umans_orca_velocities_noalloc(1, None, None, None, None, None, None, None, None, None, 129,
                                           5.0, 5.0, 0.1, 0.0, None, None)
    assert rc == 1
    assert b"exceeds the 128 ORCA lines" in lib.umans_last_error(None)
