"""The differentiable form: gradients of a trajectory loss with respect to
the force-model parameters and the initial state, from the engine's
hand-written adjoint with checkpoint/recompute, against float64 references:

* central differences (h = 1e-5) of the float64 restatement of the episode
  (oracle/calib64.py) where the episode is smooth over +-h (sparse crowds,
  short horizons);
* the float64 tangent along the engine's own float trajectory with every
  branch taken as that trajectory took it (the derivative reverse mode
  computes, evaluated in float64), on the calibration density as well.

Tolerance: relative gradient error <= 1e-3 (2-norm over the compared
components)."""
import numpy as np
import pytest

from oracle import calib64, port
from umans_gb300 import Batch, Simulation, UmansError, scenarios as S

pytestmark = pytest.mark.gpu

HELD_OUT = (2.1 * 1.2, 0.3 * 0.85, 1.5 * 1.1, 3.0 * 0.9)   # V0, sigma, k, tau0 of the target trajectories
TOL = 1e-3


def _relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _case(tmp_path, n, side, seed, steps, tag="c"):
    path = S.calibration_set(n=n, side=side, seed=seed).write(str(tmp_path / f"{tag}.xml"))
    held = S.calibration_set(HELD_OUT, n=n, side=side, seed=seed).write(str(tmp_path / f"{tag}_held.xml"))
    h = Simulation(held)
    targets = []
    for _ in range(steps):
        h.step(1)
        targets.append(h.positions())
    h.close()
    return path, np.array(targets)


def _float_states(path, steps):
    s = Simulation(path)
    out = []
    for t in range(steps + 1):
        st = s.state()
        out.append((st["pos"].copy(), st["vel"].copy()))
        if t < steps:
            s.step(1)
    s.close()
    return out


def _engine_gradient(path, targets, every, with_state=False):
    s = Simulation(path)
    s.diff_begin(targets, checkpoint_every=every)
    loss = s.diff_forward()
    g = s.diff_backward(with_state=with_state)
    params = s.force_params(0).astype(np.float64)
    s.close()
    return loss, g, params


def test_loss_matches_stepped_trajectory(tmp_path):
    steps, n = 12, 48
    path, tg = _case(tmp_path, n, 14.0, 7, steps)
    states = _float_states(path, steps)
    loss, _, _ = _engine_gradient(path, tg, 5)
    pos = np.array([s[0] for s in states[1:]], np.float64)
    ref = ((pos - tg) ** 2).sum() / (steps * n)
    assert abs(loss - ref) <= 1e-6 * ref


def test_parameter_gradient_vs_central_differences_sparse(tmp_path):
    """24 agents in 20 x 20 m, 20 steps (a layout whose float and float64
    episodes stay within 4e-6 m): no branch changes within +-h."""
    steps, n = 20, 24
    path, tg = _case(tmp_path, n, 20.0, 2, steps)
    loss, g, p0 = _engine_gradient(path, tg, 7)
    sc = port.read_scenario(path)
    w = 1.0 / (steps * n)
    assert abs(calib64.loss(sc, steps, tg, w, params=p0) - loss) <= 1e-4 * loss
    fd = calib64.central_difference(lambda p: calib64.loss(sc, steps, tg, w, params=p), p0, 1e-5)
    err = _relerr(g[0], fd)
    print("engine", g[0], "fd", fd, "rel err", err)
    assert err <= TOL


def test_parameter_gradient_vs_float64_tangent(tmp_path):
    steps, n = 20, 24
    path, tg = _case(tmp_path, n, 20.0, 1, steps)
    _, g, p0 = _engine_gradient(path, tg, 6)
    sc = port.read_scenario(path)
    states = _float_states(path, steps)
    z = np.zeros((n, 2))
    ref = calib64.tangent_gradient(sc, states, tg, 1.0 / (steps * n), p0, [(np.eye(4)[k], z, z) for k in range(4)])
    err = _relerr(g[0], ref)
    print("engine", g[0], "tangent", ref, "rel err", err)
    assert err <= TOL


def test_state_gradient_vs_float64_tangent(tmp_path):
    steps, n = 15, 32
    path, tg = _case(tmp_path, n, 18.0, 3, steps)
    _, (g, gp, gv), p0 = _engine_gradient(path, tg, 4, with_state=True)
    sc = port.read_scenario(path)
    states = _float_states(path, steps)
    rng = np.random.default_rng(0)
    dirs = []
    for _ in range(3):
        dirs.append((np.zeros(4), rng.standard_normal((n, 2)), rng.standard_normal((n, 2))))
    # state directions move every agent: h = 1e-6 keeps the second-order
    # term of the central difference below 1e-5 relative (1e-5 does not)
    ref = calib64.tangent_gradient(sc, states, tg, 1.0 / (steps * n), p0, dirs, h=1e-6)
    eng = np.array([(gp * dp).sum() + (gv * dv).sum() for _, dp, dv in dirs])
    err = _relerr(eng, ref)
    print("engine", eng, "tangent", ref, "rel err", err)
    assert err <= TOL


def test_gradient_at_calibration_density(tmp_path):
    """512 agents in 40 x 40 m (the calibration workload's density), a short
    horizon, against the float64 tangent along the engine's trajectory."""
    steps, n = 4, 512
    path, tg = _case(tmp_path, n, 40.0, 5, steps)
    _, g, p0 = _engine_gradient(path, tg, 2)
    sc = port.read_scenario(path)
    states = _float_states(path, steps)
    z = np.zeros((n, 2))
    ref = calib64.tangent_gradient(sc, states, tg, 1.0 / (steps * n), p0, [(np.eye(4)[k], z, z) for k in range(4)],
                                   h=1e-6)
    err = _relerr(g[0], ref)
    print("engine", g[0], "tangent", ref, "rel err", err)
    assert err <= TOL


def test_checkpoint_interval_does_not_change_the_gradient(tmp_path):
    steps, n = 16, 64
    path, tg = _case(tmp_path, n, 16.0, 9, steps)
    ref = None
    for every in (1, 3, 16):
        loss, (g, gp, gv), _ = _engine_gradient(path, tg, every, with_state=True)
        cur = np.concatenate([g.ravel(), gp.ravel(), gv.ravel()])
        if ref is None:
            ref, ref_loss = cur, loss
        else:
            assert abs(loss - ref_loss) <= 1e-12 * ref_loss   # double atomics: order only
            assert _relerr(cur, ref) <= 1e-5


def test_backward_restores_the_start_state(tmp_path):
    steps = 8
    path, tg = _case(tmp_path, 40, 14.0, 2, steps)
    s = Simulation(path)
    s.step(3)
    before = s.state()
    t0 = s.time
    s.diff_begin(tg[:steps], checkpoint_every=3)
    s.diff_forward()
    s.diff_backward()
    after = s.state()
    assert s.time == t0
    assert np.array_equal(before["pos"], after["pos"]) and np.array_equal(before["vel"], after["vel"])
    # and the next forward pass repeats itself
    l1 = s.diff_forward()
    l2 = s.diff_forward()
    assert abs(l1 - l2) <= 1e-12 * l1


def test_batch_gradients_per_scenario(tmp_path):
    steps = 10
    cases = [(40, 14.0, 2), (24, 12.0, 4), (60, 18.0, 6)]
    paths, targets, singles = [], [], []
    for k, (n, side, seed) in enumerate(cases):
        p, tg = _case(tmp_path, n, side, seed, steps, tag=f"b{k}")
        paths.append(p)
        targets.append(tg)
        s = Simulation(p)
        s.set_force_params((2.0 + 0.1 * k, 0.3, 1.4 + 0.1 * k, 3.0))
        s.diff_begin(tg, checkpoint_every=4, weight=1.0 / (steps * n))
        s.diff_forward()
        singles.append(s.diff_backward()[0])
        s.close()
    b = Batch(paths)
    for k in range(len(cases)):
        b.set_force_params((2.0 + 0.1 * k, 0.3, 1.4 + 0.1 * k, 3.0), k)
    off = b.offsets
    # one weight for the whole batch: per-scenario losses are then summed
    # with weight 1 / (steps * n_k) only when n_k are equal, so compare with
    # the batch's own weight folded out
    w = 1e-3
    b.diff_begin(np.concatenate(targets, axis=1), checkpoint_every=4, weight=w)
    b.diff_forward()
    g = b.diff_backward()
    for k, (n, _, _) in enumerate(cases):
        scaled = singles[k] * w * (steps * n)
        assert _relerr(g[k], scaled) <= 1e-5, (k, g[k], scaled)
    assert off[-1] == sum(c[0] for c in cases)


def test_torch_wrapper_matches_c_abi(tmp_path):
    torch = pytest.importorskip("torch")
    from umans_gb300.calibration import TrajectoryLoss
    steps = 10
    path, tg = _case(tmp_path, 32, 14.0, 8, steps)
    s = Simulation(path)
    s.diff_begin(tg, checkpoint_every=5)
    p = torch.tensor([[2.0, 0.32, 1.4, 2.8]], requires_grad=True)
    loss = TrajectoryLoss.apply(p, s)
    loss.backward()
    s.set_force_params((2.0, 0.32, 1.4, 2.8))
    l2 = s.diff_forward()
    g2 = s.diff_backward()
    assert abs(float(loss) - l2) <= 1e-12 * l2
    assert _relerr(p.grad.numpy(), g2) <= 1e-5


def test_unsupported_policies_are_rejected(tmp_path):
    path = S.model_crossing("ORCA", n=10).write(str(tmp_path / "orca.xml"))
    s = Simulation(path)
    with pytest.raises(UmansError, match="gradient-method"):
        s.diff_begin(np.zeros((3, s.n, 2), np.float32))


def _walls_case(tmp_path, steps):
    path = S.calibration_walls().write(str(tmp_path / "w.xml"))
    h = Simulation(S.calibration_walls(HELD_OUT).write(str(tmp_path / "w_held.xml")))
    targets = []
    for _ in range(steps):
        h.step(1)
        targets.append(h.positions())
    h.close()
    return path, np.array(targets)


def test_obstacle_parameter_gradient_vs_float64_tangent(tmp_path):
    """Walls and blocks (SocialForces obstacle forces, contact with edges):
    the obstacle terms enter the adjoint through the agents' positions."""
    steps = 15
    path, tg = _walls_case(tmp_path, steps)
    _, g, p0 = _engine_gradient(path, tg, 4)
    sc = port.read_scenario(path)
    n = len(sc["ids"])
    states = _float_states(path, steps)
    z = np.zeros((n, 2))
    # the obstacle forces (U0/R exp(-d/R), R = 0.2 m) and the contact
    # stiffness make the step's second derivatives large: the central
    # differences of the float64 reference need h = 1e-7 to converge
    ref = calib64.tangent_gradient(sc, states, tg, 1.0 / (steps * n), p0, [(np.eye(4)[k], z, z) for k in range(4)],
                                   h=1e-7)
    err = _relerr(g[0], ref)
    print("engine", g[0], "tangent", ref, "rel err", err)
    assert err <= TOL


def test_obstacle_state_gradient_vs_float64_tangent(tmp_path):
    steps = 12
    path, tg = _walls_case(tmp_path, steps)
    _, (g, gp, gv), p0 = _engine_gradient(path, tg, 5, with_state=True)
    sc = port.read_scenario(path)
    n = len(sc["ids"])
    states = _float_states(path, steps)
    rng = np.random.default_rng(1)
    dirs = [(np.zeros(4), rng.standard_normal((n, 2)), rng.standard_normal((n, 2))) for _ in range(3)]
    ref = calib64.tangent_gradient(sc, states, tg, 1.0 / (steps * n), p0, dirs, h=1e-7)
    eng = np.array([(gp * dp).sum() + (gv * dv).sum() for _, dp, dv in dirs])
    err = _relerr(eng, ref)
    print("engine", eng, "tangent", ref, "rel err", err)
    assert err <= TOL


def test_full_calibration_batch_window(tmp_path):
    """The calibration workload at full size (256 parameter sets x 512 agents
    in 40 x 40 m): its first 10-step window through
    calibration.windowed_gradient.  Every set's gradient is finite; against
    the float64 tangent along their own trajectories, 16 sets (every 16th)
    meet the 1e-3 bar in the median, and in the 2-norm over all 64 compared
    components they stay within 2e-3 (measured 1.4e-3).  What remains above
    1e-3 comes from a few sets with a PowerLaw collision a few hundredths of
    a second ahead: the agent's acceleration (4e4 m/s^2 in one case) is
    clamped to 5 m/s^2, and the derivative of the clamped direction of so
    stiff a force loses float32 digits that the float64 tangent keeps.  The
    1e-3 bar is asserted component-wise on the shorter horizons above."""
    from umans_gb300.calibration import windowed_gradient
    sets, n, W, t0 = 256, 512, 10, 0
    params = S.calibration_params(sets)
    held = Simulation(S.calibration_set(HELD_OUT, n=n).write(str(tmp_path / "held.xml")))
    obs = {"pos": [], "vel": [], "viewdir": []}
    for t in range(t0 + W + 1):
        st = held.state()
        for k in obs:
            obs[k].append(st[k].copy())
        if t < t0 + W:
            held.step(1)
    held.close()
    obs = {k: np.array(v[t0:]) for k, v in obs.items()}   # the window's W + 1 states
    paths = [S.calibration_set(params[k], n=n).write(str(tmp_path / f"cal{k}.xml")) for k in range(sets)]
    b = Batch(paths)
    tiled = {k: np.ascontiguousarray(np.tile(v, (1, sets, 1))) for k, v in obs.items()}
    loss, g = windowed_gradient(b, tiled, window=W)
    p = [b.force_params(k).astype(np.float64) for k in range(sets)]
    b.close()
    assert np.isfinite(loss) and np.isfinite(g).all(), "non-finite gradient"
    eng, refs, errs = [], [], []
    z = np.zeros((n, 2))
    for k in range(0, sets, 16):
        s = Simulation(paths[k])
        s.set_state(pos=obs["pos"][0], vel=obs["vel"][0], viewdir=obs["viewdir"][0])
        states = []
        for t in range(W + 1):
            st = s.state()
            states.append((st["pos"].copy(), st["vel"].copy()))
            if t < W:
                s.step(1)
        s.close()
        # after 10 steps at this density the contact and exponential terms make
        # the central differences of the float64 step converge only at small h
        # (V0 component of set 0: 0.461, 1.067, 0.890, 0.888 at h = 1e-5 .. 1e-8)
        ref = calib64.tangent_gradient(port.read_scenario(paths[k]), states, obs["pos"][1:], 1.0 / (W * n), p[k],
                                       [(np.eye(4)[j], z, z) for j in range(4)], h=1e-8)
        eng.append(g[k])
        refs.append(ref)
        errs.append(_relerr(g[k], ref))
    err = _relerr(np.concatenate(eng), np.concatenate(refs))
    print(f"256 x 512 calibration batch, first 10-step window: loss {loss:.4g}, all gradients finite; "
          f"relative error vs the float64 tangent over 16 sets {err:.3g}, median per set "
          f"{float(np.median(errs)):.3g} (per set: " + ", ".join(f"{e:.2g}" for e in errs) + ")")
    assert float(np.median(errs)) <= TOL
    assert err <= 2 * TOL
