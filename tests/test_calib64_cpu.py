"""The float64 restatement used by the gradient checks (oracle/calib64.py),
pinned against the bit-exact float port of the reference: one step from the
same float state agrees to float rounding, and the first steps of an episode
stay within 1e-5 m.  Its tangent (branches frozen) agrees with central
differences of the episode where the episode is smooth."""
import numpy as np

from oracle import calib64, port
from umans_gb300 import scenarios as S


def _read(tmp_path, n, side, seed, params=None, tag="c"):
    return port.read_scenario(S.calibration_set(params, n=n, side=side, seed=seed).write(str(tmp_path / f"{tag}.xml")))


def test_single_steps_match_the_port(tmp_path):
    sc = _read(tmp_path, 128, 20.0, 5)
    pols = calib64.policy_arrays(sc)
    P = port.PortSim(sc)
    worst = 0.0
    for _ in range(12):
        st0 = P.state()
        P.step(1)
        st = P.state()
        p, v = calib64.step(sc, pols, st0["pos"].astype(np.float64), st0["vel"].astype(np.float64))
        worst = max(worst, float(np.abs(p - st["pos"]).max()))
    # float rounding of the port, amplified by PowerLaw's cancellation near
    # small relative speeds
    assert worst <= 1e-4


def test_sparse_episode_matches_the_port(tmp_path):
    sc = _read(tmp_path, 24, 20.0, 2)
    P = port.PortSim(sc)
    ref = []
    for _ in range(20):
        P.step(1)
        ref.append(P.state()["pos"].copy())
    traj = calib64.episode(sc, 20)
    assert np.abs(traj - np.array(ref)).max() <= 1e-5


def test_tangent_matches_central_differences_when_smooth(tmp_path):
    steps, n = 20, 24
    sc = _read(tmp_path, n, 20.0, 2)
    held = _read(tmp_path, n, 20.0, 2, params=(2.52, 0.255, 1.65, 2.7), tag="h")
    tg = calib64.episode(held, steps)
    p0 = np.array([2.1, 0.3, 1.5, 3.0], np.float32).astype(np.float64)
    w = 1.0 / (steps * n)
    # the float64 episode's own trajectory as the "float" trajectory
    pols = calib64.policy_arrays(sc)
    pos, vel = sc["pos"].astype(np.float64), np.zeros((n, 2))
    states = [(pos, vel)]
    for _ in range(steps):
        pos, vel = calib64.step(sc, pols, pos, vel, p0)
        states.append((pos, vel))
    z = np.zeros((n, 2))
    tan = calib64.tangent_gradient(sc, states, tg, w, p0, [(np.eye(4)[k], z, z) for k in range(4)])
    fd = calib64.central_difference(lambda p: calib64.loss(sc, steps, tg, w, params=p), p0, 1e-5)
    assert np.linalg.norm(tan - fd) <= 1e-4 * np.linalg.norm(fd)


def test_obstacle_steps_match_the_port(tmp_path):
    """Walls and blocks: SocialForces obstacle forces and contact with edges."""
    sc = port.read_scenario(S.calibration_walls().write(str(tmp_path / "w.xml")))
    assert len(sc["edges"]) == 40
    pols = calib64.policy_arrays(sc)
    P = port.PortSim(sc)
    worst = 0.0
    for _ in range(30):
        st0 = P.state()
        P.step(1)
        st = P.state()
        p, v = calib64.step(sc, pols, st0["pos"].astype(np.float64), st0["vel"].astype(np.float64))
        worst = max(worst, float(np.abs(p - st["pos"]).max()))
    assert worst <= 1e-4
