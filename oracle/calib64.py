"""FP64 restatement of the force-based step, for checking the differentiable
form's gradients.

TEST INFRASTRUCTURE ONLY: the gradient tests and bench.py's check of the
differentiable form use this module; the product never imports it.

One step, for scenarios whose agents share one policy that uses the
gradient method with SocialForcesAvoidance, PowerLaw and GoalReachingForce
costs, in an infinite world, evaluated in float64 over pair lists:

* preferred velocity: Agent::ComputePreferredVelocity (src/Engine/core/agent.cpp:52-59),
  zero once |goal - pos| <= radius (agent.cpp:99-102);
* neighbours: every other agent within the policy's interaction range
  (Policy::getInteractionRange, src/Engine/core/policy.cpp:34-41; the kd-tree
  query of src/Engine/core/worldInfinite.cpp:31-52), each cost then keeping
  those within its own range (ObjectInteractionForces::ComputeForce,
  src/Engine/CostFunctions/ObjectInteractionForces.cpp:26-48);
* forces: SocialForcesAvoidance::ComputeAgentInteractionForce
  (src/Engine/CostFunctions/SocialForcesAvoidance.cpp:26-110),
  PowerLaw::ComputeAgentInteractionForce (src/Engine/CostFunctions/PowerLaw.cpp:28-66),
  GoalReachingForce (src/Engine/CostFunctions/GoalReachingForce.cpp:26-29);
* velocity: Policy::getAccelerationFromGradient (policy.cpp:78-89) with
  ForceBasedFunction::GetGradient (src/Engine/CostFunctions/ForceBasedFunction.cpp:32-36),
  i.e. a = sum_c coeff_c F_c / mass_c, clamped to the maximum acceleration,
  new velocity clamped to the maximum speed; zero at the goal
  (Policy::ComputeNewVelocity, policy.cpp:43-76);
* contact forces: Policy::getContactForces (policy.cpp:107-141), with the
  obstacle edges as well;
* static obstacles: each agent's edges within the policy's range
  (WorldBase::computeNeighboringObstacles, worldBase.cpp:62-77), the
  SocialForces obstacle force (SocialForcesAvoidance.cpp:112-140) and
  contact with edges (policy.cpp:126-137), the nearest point of an edge as
  nearestPointOnLine with onSegment (vector2D.h:274-296);
* integration: Agent::UpdateVelocityAndPosition (agent.cpp:71-93), contact
  acceleration = force / 80.

The step is piecewise smooth: neighbour sets, the force models' cut-offs,
the view-angle factor, the clamps and the contact test are branches.  With
``branches`` (recorded by ``record_branches`` from a float trajectory) every
branch is taken as recorded and the map is smooth in the parameters and the
initial state: central differences of it give the derivative on the piece
the float trajectory lies in, which is what the engine's adjoint computes.
Without, branches are evaluated on the float64 state (the view-angle test
as the reference's float angle() evaluates it).
"""
from __future__ import annotations

import numpy as np

K_SF, K_PL, K_GR = 2, 3, 4   # CostKind values of the port and the engine
VIEW_HALF = 100.0 * np.pi / 180.0


def policy_arrays(sc: dict):
    """Policy data of a scenario read by oracle.port.read_scenario."""
    out = []
    for P in sc["policies"]:
        if P.method != 0:
            raise ValueError("gradient-method policies only")
        costs = []
        for c in range(P.ncost):
            C = P.cost[c]
            if C.kind not in (K_SF, K_PL, K_GR):
                raise ValueError("SocialForcesAvoidance, PowerLaw and GoalReachingForce only")
            costs.append(dict(kind=C.kind, coeff=float(C.coeff), range=float(C.range),
                              p=[float(C.p[k]) for k in range(8)]))
        rng = max([float(P.cost[c].range) for c in range(P.ncost)] + [0.0])
        out.append(dict(relax=float(P.relax_time), contact=float(P.contact_scale), costs=costs, range=rng))
    if len(set(np.asarray(sc["policy_index"]).tolist())) > 1:
        raise ValueError("one policy for all agents")
    return out


def _view_less(pos, vel, I, J):
    """angle(vel_i, p_j - p_i) < 100 degrees per pair, evaluated as the
    reference's float angle() does (src/Engine/tools/vector2D.h:176-190):
    float magnitudes and dot product, the quotient in double, and angle 0
    for zero lengths or a quotient outside [-1, 1] (nearly opposite
    vectors)."""
    f = np.float32
    p = pos.astype(f)
    a = vel.astype(f)[I]
    b = p[J] - p[I]
    ma = np.sqrt(a[:, 0] * a[:, 0] + a[:, 1] * a[:, 1])
    mb = np.sqrt(b[:, 0] * b[:, 0] + b[:, 1] * b[:, 1])
    lengths = (ma * mb).astype(np.float64)
    dot = (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]).astype(np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        frac = dot / np.where(lengths == 0, 1.0, lengths)
    ang = np.where((lengths == 0) | (frac < -1) | (frac > 1), 0.0,
                   np.arccos(np.clip(frac, -1.0, 1.0)).astype(f))
    return ang < f(VIEW_HALF)


def _norm(v):
    return np.sqrt((v * v).sum(-1))


def _sum_to(I, f, n):
    return np.stack([np.bincount(I, weights=f[:, 0], minlength=n),
                     np.bincount(I, weights=f[:, 1], minlength=n)], 1)


def _clamp(v, L, flag):
    m = _norm(v)
    return np.where(flag[:, None], v / np.where(m > 0, m, 1.0)[:, None] * L[:, None], v)


def _edge_regime(p, a, b):
    """0: nearest point interior, 1: end a (k >= 1), 2: end b (k <= 0), 3:
    point-like edge (a == b)."""
    line = a - b
    L2 = (line * line).sum(-1)
    k = ((p - b) * line).sum(-1) / np.where(L2 > 0, L2, 1.0)
    reg = np.where(k >= 1, 1, np.where(k <= 0, 2, 0))
    return np.where(L2 > 0, reg, 3)


def _edge_diff(p, a, b, reg):
    """p - nearest point of the edge, the nearest point's regime given."""
    line = a - b
    L2 = (line * line).sum(-1)
    k = ((p - b) * line).sum(-1) / np.where(L2 > 0, L2, 1.0)
    k = np.where(reg == 0, k, np.where(reg == 1, 1.0, 0.0))
    nearest = np.where((reg == 3)[:, None], a, a * k[:, None] + b * (1 - k)[:, None])
    return p - nearest


def step(sc: dict, pols, pos, vel, params=None, branches=None, record=None):
    """One step in float64 from (pos, vel).  params = (V0, sigma, k, tau0)
    overriding the policy's values, or None.  branches: a dict made by
    ``record_branches`` for this step (taken as recorded); record: a dict
    that receives this step's branch decisions.  Returns (pos, vel)."""
    if sc["world"] != 0:
        raise ValueError("infinite worlds only")
    P = pols[0]
    n = pos.shape[0]
    dt = float(sc["dt"])
    radius = sc["radius"].astype(np.float64)
    prefs = sc["pref_speed"].astype(np.float64)
    maxs = sc["max_speed"].astype(np.float64)
    maxa = sc["max_accel"].astype(np.float64)
    goal = sc["goal"].astype(np.float64)
    B = branches
    R_ = {} if record is None else record
    w = goal - pos
    at_goal = B["at_goal"] if B else (w * w).sum(-1) <= radius ** 2
    dw = _norm(w)
    pref = np.where(at_goal[:, None], 0.0, w / np.where(dw > 0, dw, 1.0)[:, None] * prefs[:, None])
    # the neighbour's goal direction and speed (SocialForcesAvoidance.cpp:58-59)
    pn = _norm(pref)
    ebj = np.where((pn > 0)[:, None], pref / np.where(pn > 0, pn, 1.0)[:, None], 0.0)
    vbj = _norm(vel)
    if B:
        I, J = B["I"], B["J"]
    else:
        D2 = ((pos[:, None, :] - pos[None, :, :]) ** 2).sum(-1)
        nb = (D2 <= P["range"] ** 2) & ~np.eye(n, dtype=bool)
        I, J = np.nonzero(nb)
    R_["at_goal"], R_["I"], R_["J"] = at_goal, I, J
    X = pos[I] - pos[J]
    d2 = (X * X).sum(-1)
    rsum = radius[I] + radius[J]
    # obstacle edges within the policy's range, per agent
    edges = np.asarray(sc.get("edges", np.zeros((0, 4))), np.float64).reshape(-1, 4)
    if len(edges):
        if B:
            Io, Eo, reg = B["Io"], B["Eo"], B["reg"]
        else:
            ii, ee = np.meshgrid(np.arange(n), np.arange(len(edges)), indexing="ij")
            ii, ee = ii.ravel(), ee.ravel()
            rg = _edge_regime(pos[ii], edges[ee, :2], edges[ee, 2:])
            dd = _edge_diff(pos[ii], edges[ee, :2], edges[ee, 2:], rg)
            sel = (dd * dd).sum(-1) <= P["range"] ** 2
            Io, Eo, reg = ii[sel], ee[sel], rg[sel]
        R_["Io"], R_["Eo"], R_["reg"] = Io, Eo, reg
        odiff = _edge_diff(pos[Io], edges[Eo, :2], edges[Eo, 2:], reg)
        od2 = (odiff * odiff).sum(-1)
        odist = np.sqrt(od2)
    acc = np.zeros_like(vel)
    for ci, c in enumerate(P["costs"]):
        if c["kind"] == K_GR:
            F = (pref - vel) / max(P["relax"], dt)
        else:
            inr = B[f"inr{ci}"] if B else d2 <= c["range"] ** 2
            R_[f"inr{ci}"] = inr
            with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
                if c["kind"] == K_SF:
                    dtp = c["p"][0]
                    V0 = params[0] if params is not None else c["p"][1]
                    sigma = params[1] if params is not None else c["p"][2]
                    magR = np.sqrt(d2)
                    Vv = ebj[J] * (vbj[J] * dtp)[:, None]
                    magV = _norm(Vv)
                    R2 = X - Vv
                    magR2 = _norm(R2)
                    T = vbj[J] * dtp
                    bSq = (magR + magR2) ** 2 - T ** 2
                    b = 0.5 * np.sqrt(np.abs(bSq))
                    ok = B[f"ok{ci}"] if B else (magR > rsum) & (bSq > 0) & (b >= 0.001)
                    scale = B[f"scale{ci}"] if B else np.where(_view_less(pos, vel, I, J), 1.0, 0.5)
                    lens = magR * magV
                    cth = np.where(lens > 0, (X * Vv).sum(-1) / np.where(lens > 0, lens, 1.0), 0.0)
                    dmagR2 = (magR - magV * cth) / magR2
                    db = 2 * (magR + magR2) * (1 + dmagR2) / (8 * b)
                    dV = -V0 / sigma * np.exp(-b / sigma) * db
                    f = -X * (dV * scale)[:, None]
                    R_[f"scale{ci}"] = scale
                else:
                    k = params[2] if params is not None else c["p"][0]
                    tau0 = params[3] if params is not None else c["p"][1]
                    v = vel[I] - vel[J]
                    a = (v * v).sum(-1)
                    bb = -(X * v).sum(-1)
                    cc = d2 - rsum ** 2
                    d = bb * bb - a * cc
                    sd = np.sqrt(np.abs(d))
                    tau = (bb - sd) / a
                    ok = B[f"ok{ci}"] if B else (cc > 0) & (d > 0) & (tau >= 0.001) & (tau <= tau0)
                    comp1 = -k * np.exp(-tau / tau0) * (2 / tau + 1 / tau0) / (a * tau * tau)
                    comp2 = v - (X * a[:, None] + v * bb[:, None]) / sd[:, None]
                    f = comp2 * comp1[:, None]
            R_[f"ok{ci}"] = ok
            use = inr & ok
            F = _sum_to(I[use], f[use], n)
            if c["kind"] == K_SF and len(edges):
                oinr = B[f"oinr{ci}"] if B else od2 <= c["range"] ** 2
                ook = B[f"ook{ci}"] if B else odist >= 0.001
                R_[f"oinr{ci}"], R_[f"ook{ci}"] = oinr, ook
                U0, Rr = c["p"][3], c["p"][4]
                fo = odiff * (U0 / Rr * np.exp(-odist / Rr))[:, None]
                uo = oinr & ook
                F = F + _sum_to(Io[uo], fo[uo], n)
        acc += c["coeff"] * F / c["p"][5]
    acl = B["acl"] if B else _norm(acc) > maxa
    acc = _clamp(acc, maxa, acl)
    u = vel + acc * dt
    spd = B["spd"] if B else _norm(u) > maxs
    u = _clamp(u, maxs, spd)
    u = np.where(at_goal[:, None], 0.0, u)
    R_["acl"], R_["spd"] = acl, spd
    contact = np.zeros_like(vel)
    if P["contact"] > 0:
        md = np.sqrt(d2)
        inter = rsum - md
        take = B["take"] if B else (inter > 0) & (md > 0)
        R_["take"] = take
        f = X[take] / md[take][:, None] * (P["contact"] * inter[take])[:, None]
        contact = _sum_to(I[take], f, n)
        if len(edges):
            ointer = radius[Io] - odist
            otake = B["otake"] if B else (ointer > 0) & (odist > 0)
            R_["otake"] = otake
            fo = odiff[otake] / odist[otake][:, None] * (P["contact"] * ointer[otake])[:, None]
            contact = contact + _sum_to(Io[otake], fo, n)
    vel2 = u + contact / 80.0 * dt
    return pos + vel2 * dt, vel2


def record_branches(sc: dict, states):
    """Branch decisions of each step of a float trajectory: states[t] =
    (pos, vel) at the start of step t (float32 arrays)."""
    pols = policy_arrays(sc)
    out = []
    for pos, vel in states:
        rec = {}
        step(sc, pols, np.asarray(pos, np.float64), np.asarray(vel, np.float64), record=rec)
        out.append(rec)
    return out


def episode(sc: dict, steps: int, params=None, pos0=None, vel0=None, branches=None):
    """Positions after each of `steps` steps: (steps, n, 2) float64."""
    pols = policy_arrays(sc)
    pos = np.asarray(sc["pos"] if pos0 is None else pos0, np.float64)
    vel = np.zeros_like(pos) if vel0 is None else np.asarray(vel0, np.float64)
    out = np.empty((steps,) + pos.shape)
    for t in range(steps):
        pos, vel = step(sc, pols, pos, vel, params, None if branches is None else branches[t])
        out[t] = pos
    return out


def loss(sc: dict, steps: int, targets, weight: float, params=None, pos0=None, vel0=None,
         branches=None) -> float:
    """weight * sum_t sum_i |p_i(t) - target_i(t)|^2 in float64."""
    traj = episode(sc, steps, params, pos0, vel0, branches)
    return float(weight * ((traj - np.asarray(targets, np.float64)) ** 2).sum())


def central_difference(f, x, h: float = 1e-5):
    """Central differences of a scalar function at x (float64 array)."""
    x = np.asarray(x, np.float64)
    g = np.empty_like(x)
    for k in range(x.size):
        e = np.zeros_like(x)
        e.flat[k] = h
        g.flat[k] = (f(x + e) - f(x - e)) / (2 * h)
    return g


def tangent_gradient(sc: dict, states, targets, weight: float, params, directions, h: float = 1e-5):
    """Directional derivatives of the loss along a float trajectory.

    states[t] = (pos, vel) at the start of step t, t = 0..steps (float32;
    states[steps] is the final state); the loss is
    weight * sum_{t=1..steps} sum_i |pos_t - target_{t-1}|^2 on those states.
    Each direction is (dparams[4], dpos0[n, 2], dvel0[n, 2]); the tangent of
    the state is carried step by step with central differences (step h) of
    the float64 step at the recorded state, every branch taken as the float
    trajectory took it.  This is the derivative that reverse mode along the
    same trajectory computes, in float64."""
    pols = policy_arrays(sc)
    steps = len(states) - 1
    br = record_branches(sc, states[:steps])
    p = np.asarray(params, np.float64)
    out = []
    for dth, dp0, dv0 in directions:
        dth = np.asarray(dth, np.float64)
        tp = np.asarray(dp0, np.float64)
        tv = np.asarray(dv0, np.float64)
        g = 0.0
        for t in range(steps):
            pos = np.asarray(states[t][0], np.float64)
            vel = np.asarray(states[t][1], np.float64)
            a = step(sc, pols, pos + h * tp, vel + h * tv, p + h * dth, br[t])
            b = step(sc, pols, pos - h * tp, vel - h * tv, p - h * dth, br[t])
            tp = (a[0] - b[0]) / (2 * h)
            tv = (a[1] - b[1]) / (2 * h)
            r = np.asarray(states[t + 1][0], np.float64) - np.asarray(targets[t], np.float64)
            g += 2 * weight * float((r * tp).sum())
        out.append(g)
    return np.array(out)
