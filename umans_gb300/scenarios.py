"""Seeded scenario generators written as UMANS scenario XML.

Every workload is written in the reference's own scenario format
(``<Simulation>/<World>/<Policies>/<Agents>``, parsed by
``CrowdSimulator::FromConfigFile``, src/Engine/core/crowdSimulator.cpp:516-647),
so the same file drives the reference CPU engine, the CPU oracle and this
engine.  Coordinates are written with 9 significant digits, which round-trips
every float32 value exactly through ``strtof``.

Workloads (agent counts can be reduced for tests with ``n=``):

* ``circle_orca``          50 agents on a circle of radius 25 m, antipodal goals,
                           ORCA (global method, range 8, time horizon 5), dt 0.1.
* ``socialforces_toric``   100k agents uniform in a 400x400 m toric world,
                           SocialForcesAvoidance(range 5) + GoalReachingForce,
                           gradient method, dt 0.1.
* ``karamouzas_corridor``  two opposing flows on a jittered 1 m lattice,
                           Karamouzas(range 10), regular sampling 10 speeds x 20
                           angles + base = 181 samples, dt 0.05.
* ``batch_mixed``          4096 independent scenarios, agent counts log-uniform in
                           [8, 2048], circle / random-square layouts, policies
                           cycling ORCA / PowerLaw-sampling / SocialForces-gradient.
* ``calibration_set``      512 agents in a 40x40 m square with one parameter set of
                           SocialForcesAvoidance + PowerLaw + GoalReachingForce.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np


def _f(x) -> str:
    return "%.9g" % float(np.float32(x))


ORCA_POLICY = (
    '<Policy id="{pid}" OptimizationMethod="global" RelaxationTime="0">'
    '<costfunction name="ORCA" range="8" timeHorizon="5"/></Policy>')

SF_POLICY = (
    '<Policy id="{pid}" OptimizationMethod="gradient" RelaxationTime="0.5">'
    '<costfunction name="SocialForcesAvoidance" range="5"{sfparams}/>'
    '<costfunction name="GoalReachingForce"/></Policy>')

POWERLAW_SAMPLING_POLICY = (
    '<Policy id="{pid}" OptimizationMethod="sampling" SamplingType="regular" '
    'SamplingBase="zero" SamplingBaseDirection="unit" SamplingAngle="360" '
    'SpeedSamples="4" AngleSamples="36" SamplingRadius="maximum speed" '
    'RelaxationTime="0.5">'
    '<costfunction name="PowerLaw" range="5"/>'
    '<costfunction name="GoalReachingForce"/></Policy>')

KARAMOUZAS_POLICY = (
    '<Policy id="{pid}" OptimizationMethod="sampling" SamplingType="regular" '
    'SamplingBase="zero" SamplingBaseDirection="preferred velocity" '
    'SamplingAngle="180" SpeedSamples="10" AngleSamples="20" '
    'IncludeBaseAsSample="true" SamplingRadius="maximum speed" RelaxationTime="0">'
    '<costfunction name="Karamouzas" range="10"/></Policy>')

CALIBRATION_POLICY = (
    '<Policy id="{pid}" OptimizationMethod="gradient" RelaxationTime="0.5">'
    '<costfunction name="SocialForcesAvoidance" range="5" V0="{V0}" sigma="{sigma}"/>'
    '<costfunction name="PowerLaw" range="5" k="{k}" tau0="{tau0}"/>'
    '<costfunction name="GoalReachingForce"/></Policy>')


@dataclass
class Scenario:
    """A scenario in memory: world, policies (XML snippets) and agents."""
    dt: float
    world: str                      # "Infinite" or "Toric"
    width: float = 0.0
    height: float = 0.0
    end_time: float | None = None
    policies: list = field(default_factory=list)   # <Policy> XML strings or policy.Policy objects
    pos: np.ndarray = None          # (n, 2) float32
    goal: np.ndarray = None         # (n, 2) float32
    radius: np.ndarray = None       # (n,) float32
    pref_speed: np.ndarray = None   # (n,) float32
    max_speed: np.ndarray = None    # (n,) float32
    policy_id: np.ndarray = None    # (n,) int
    obstacles: list = field(default_factory=list)   # polygons: (k, 2) vertex arrays
    start_time: np.ndarray = None   # (n,) float32 or None: timed insertion (s)
    remove_at_goal: np.ndarray = None   # (n,) bool or None

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def to_xml(self) -> str:
        obs = ""
        if self.obstacles:
            obs = "<Obstacles>" + "".join(
                "<Obstacle>" + "".join(f'<Point x="{_f(x)}" y="{_f(y)}"/>' for x, y in np.asarray(poly, np.float32))
                + "</Obstacle>" for poly in self.obstacles) + "</Obstacles>"
        w = (f'<World type="Toric" width="{_f(self.width)}" height="{_f(self.height)}">{obs}</World>'
             if self.world == "Toric" else f'<World type="Infinite">{obs}</World>')
        end = f' end_time="{_f(self.end_time)}"' if self.end_time is not None else ""
        out = ['<?xml version="1.0" encoding="utf-8"?>',
               f'<Simulation delta_time="{_f(self.dt)}"{end}>', w,
               "<Policies>", *(p if isinstance(p, str) else p.to_xml() for p in self.policies),
               "</Policies>", "<Agents>"]
        for i in range(self.n):
            extra = ""
            if self.start_time is not None and self.start_time[i] != 0:
                extra += f' start_time="{_f(self.start_time[i])}"'
            if self.remove_at_goal is not None and self.remove_at_goal[i]:
                extra += ' remove_at_goal="true"'
            out.append(
                f'<Agent rad="{_f(self.radius[i])}" pref_speed="{_f(self.pref_speed[i])}" '
                f'max_speed="{_f(self.max_speed[i])}"{extra}>'
                f'<pos x="{_f(self.pos[i, 0])}" y="{_f(self.pos[i, 1])}"/>'
                f'<goal x="{_f(self.goal[i, 0])}" y="{_f(self.goal[i, 1])}"/>'
                f'<Policy id="{int(self.policy_id[i])}"/></Agent>')
        out += ["</Agents>", "</Simulation>", ""]
        return "\n".join(out)

    def write(self, path: str) -> str:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "w") as fh:
            fh.write(self.to_xml())
        return path


def _agents(n, pos, goal, radius=0.3, pref=1.3, maxs=1.8, pid=0):
    f32 = np.float32
    return dict(pos=np.asarray(pos, f32).reshape(n, 2),
                goal=np.asarray(goal, f32).reshape(n, 2),
                radius=np.full(n, radius, f32) if np.isscalar(radius) else np.asarray(radius, f32),
                pref_speed=np.full(n, pref, f32) if np.isscalar(pref) else np.asarray(pref, f32),
                max_speed=np.full(n, maxs, f32) if np.isscalar(maxs) else np.asarray(maxs, f32),
                policy_id=np.full(n, pid, np.int64) if np.isscalar(pid) else np.asarray(pid, np.int64))


def circle_orca(n: int = 50, radius_m: float = 25.0, steps: int = 300) -> Scenario:
    """n agents evenly spaced on a circle, goals at the antipodal points, ORCA."""
    ang = 2.0 * np.pi * np.arange(n) / n
    pos = np.stack([radius_m * np.cos(ang), radius_m * np.sin(ang)], 1)
    return Scenario(dt=0.1, world="Infinite", end_time=steps * 0.1,
                    policies=[ORCA_POLICY.format(pid=0)],
                    **_agents(n, pos, -pos))


def socialforces_toric(n: int = 100_000, side: float = 400.0, seed: int = 2,
                       density: float | None = None) -> Scenario:
    """Uniform agents and goals in a toric square; SocialForces + goal force.

    ``density`` (agents per m^2), when given, overrides ``side`` so that a
    reduced ``n`` keeps the neighbourhood size of the full workload
    (100k agents in 400x400 m = 0.625 agents/m^2).
    """
    if density is not None:
        side = math.sqrt(n / density)
    rng = np.random.default_rng(seed)
    h = side / 2.0
    pos = rng.uniform(-h, h, (n, 2))
    goal = rng.uniform(-h, h, (n, 2))
    pref = np.clip(rng.normal(1.3, 0.1, n), 0.8, 1.8)
    return Scenario(dt=0.1, world="Toric", width=side, height=side,
                    policies=[SF_POLICY.format(pid=0, sfparams="")],
                    **_agents(n, pos, goal, pref=pref))


def karamouzas_corridor(n: int = 1_000_000, width: float = 100.0, seed: int = 3) -> Scenario:
    """Two opposing flows on a jittered 1 m lattice (1 agent/m^2).

    The corridor is ``width`` m high and as long as needed for n agents at one
    agent per m^2; the left half walks to x=+L/2, the right half to x=-L/2.
    """
    rng = np.random.default_rng(seed)
    rows = int(width)
    cols = int(math.ceil(n / rows))
    length = float(cols)
    xs = -length / 2 + 0.5 + np.arange(cols)
    ys = -width / 2 + 0.5 + np.arange(rows)
    gx, gy = np.meshgrid(xs, ys, indexing="ij")
    pos = np.stack([gx.ravel(), gy.ravel()], 1)[:n]
    pos = pos + rng.uniform(-0.25, 0.25, pos.shape)
    left = pos[:, 0] < 0
    goal = pos.copy()
    goal[:, 0] = np.where(left, length / 2, -length / 2)
    return Scenario(dt=0.05, world="Infinite",
                    policies=[KARAMOUZAS_POLICY.format(pid=0)],
                    **_agents(n, pos, goal))


def batch_counts(num: int = 4096, seed: int = 4, lo: int = 8, hi: int = 2048) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), num))).astype(np.int64)


def batch_member(k: int, n: int, seed: int = 4) -> Scenario:
    """Scenario k of the mixed batch: layout alternates circle / random square,
    policy cycles ORCA / PowerLaw-sampling / SocialForces-gradient."""
    rng = np.random.default_rng([seed, k])
    if k % 2 == 0:
        r = max(n * 1.5 / (2 * math.pi), 2.0)
        ang = 2.0 * np.pi * np.arange(n) / n
        pos = np.stack([r * np.cos(ang), r * np.sin(ang)], 1)
        # small jitter: exact distance ties on a symmetric circle are ordered
        # by the reference's kd-tree traversal, which nothing else reproduces
        pos = pos + rng.uniform(-0.01, 0.01, pos.shape)
        goal = -pos
    else:
        side = math.sqrt(n / 0.5)
        pos = rng.uniform(-side / 2, side / 2, (n, 2))
        goal = rng.uniform(-side / 2, side / 2, (n, 2))
    kind = k % 3
    pol = [ORCA_POLICY, POWERLAW_SAMPLING_POLICY, SF_POLICY][kind].format(pid=0, sfparams="")
    return Scenario(dt=0.1, world="Infinite", policies=[pol], **_agents(n, pos, goal))


DEFAULT_CALIBRATION = dict(V0=2.1, sigma=0.3, k=1.5, tau0=3.0)


def calibration_params(sets: int = 256, seed: int = 5) -> np.ndarray:
    """(sets, 4) float32 parameters (V0, sigma, k, tau0), each within +-30% of default."""
    rng = np.random.default_rng(seed)
    base = np.array([DEFAULT_CALIBRATION[k] for k in ("V0", "sigma", "k", "tau0")], np.float64)
    return (base * rng.uniform(0.7, 1.3, (sets, 4))).astype(np.float32)


def calibration_set(params=None, n: int = 512, side: float = 40.0, seed: int = 5) -> Scenario:
    """One parameter set of the calibration workload (shared seeded layout)."""
    p = DEFAULT_CALIBRATION if params is None else dict(zip(("V0", "sigma", "k", "tau0"), map(float, params)))
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-side / 2, side / 2, (n, 2))
    goal = rng.uniform(-side / 2, side / 2, (n, 2))
    pol = CALIBRATION_POLICY.format(pid=0, **{k: _f(v) for k, v in p.items()})
    return Scenario(dt=0.1, world="Infinite", policies=[pol], **_agents(n, pos, goal))


def calibration_walls(params=None, n: int = 48, side: float = 16.0, seed: int = 6) -> Scenario:
    """A calibration parameter set in a walled square with a few blocks (the
    differentiable form with static obstacles): the square's four walls just
    outside the agents' area (four agents start touching them), and 6 blocks
    inside it."""
    sc = calibration_set(params, n=n, side=side, seed=seed)
    h = side / 2 + 0.6
    sc.pos[:4] = np.array([[h - 0.2, 1.0], [-h + 0.2, -1.0], [2.0, h - 0.25], [-2.0, -h + 0.25]], np.float32)
    t = 0.4
    sc.obstacles = [np.array(q, np.float32) for q in (
        [[-h - t, -h - t], [h + t, -h - t], [h + t, -h], [-h - t, -h]],
        [[-h - t, h], [h + t, h], [h + t, h + t], [-h - t, h + t]],
        [[-h - t, -h], [-h, -h], [-h, h], [-h - t, h]],
        [[h, -h], [h + t, -h], [h + t, h], [h, h]])]
    rng = np.random.default_rng(seed + 100)
    sc.obstacles += block_field(6, side - 2.0, rng, size=(0.6, 1.2), keep_clear=sc.pos)
    return sc


# The policy configurations the reference ships, one per navigation model
# (parameter values as in the reference's examples/policies/*.xml; the same
# values are needed for trajectories to be comparable).
MODEL_POLICIES = {
    "ORCA": '<Policy id="0" OptimizationMethod="global" RelaxationTime="0">'
            '<costfunction range="5" name="ORCA"/></Policy>',
    "RVO": '<Policy id="0" OptimizationMethod="sampling" SamplingType="random" SamplingBase="current velocity" '
           'SamplingBaseDirection="unit" SamplingAngle="360" RandomSamples="250" '
           'SamplingRadius="maximum acceleration" RelaxationTime="0">'
           '<costfunction range="5" name="RVO"/></Policy>',
    "SocialForces": '<Policy id="0" OptimizationMethod="gradient" RelaxationTime="0.5">'
                    '<costfunction range="5" name="SocialForcesAvoidance"/>'
                    '<costfunction name="GoalReachingForce"/></Policy>',
    "PowerLaw": '<Policy id="0" OptimizationMethod="gradient" RelaxationTime="0.5">'
                '<costfunction range="5" name="PowerLaw"/><costfunction name="GoalReachingForce"/></Policy>',
    "Karamouzas": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
                  'SamplingBaseDirection="preferred velocity" SamplingAngle="180" SpeedSamples="15" '
                  'AngleSamples="19" SamplingRadius="maximum speed" RelaxationTime="0" IncludeBaseAsSample="true">'
                  '<costfunction range="5" name="Karamouzas"/></Policy>',
    "Moussaid": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
                'SamplingBaseDirection="preferred velocity" SamplingAngle="180" SpeedSamples="5" '
                'AngleSamples="19" SamplingRadius="preferred speed" RelaxationTime="0.5">'
                '<costfunction range="5" name="Moussaid"/></Policy>',
    "VanToll": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
               'SamplingBaseDirection="preferred velocity" SamplingAngle="180" SpeedSamples="2" '
               'AngleSamples="19" SamplingRadius="preferred speed" RelaxationTime="0.25">'
               '<costfunction range="5" name="VanToll"/></Policy>',
    "PLEdestrians": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
                    'SamplingBaseDirection="unit" SamplingAngle="360" SpeedSamples="4" AngleSamples="36" '
                    'SamplingRadius="maximum speed" RelaxationTime="0.5">'
                    '<costfunction range="5" name="PLEdestrians" t_min="0.5" t_max="3"/></Policy>',
    "Paris": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
             'SamplingBaseDirection="unit" SamplingAngle="360" SpeedSamples="4" AngleSamples="36" '
             'SamplingRadius="maximum speed" RelaxationTime="0">'
             '<costfunction range="5" name="Paris"/></Policy>',
    "Dutra": '<Policy id="0" OptimizationMethod="gradient">'
             '<costfunction coeff="20" range="5" name="TtcaDca" sigmaTtca="1" sigmaDca="0.3" '
             'sigmaAngle_goal="2" sigmaSpeed_goal="2"/></Policy>',
    "FOEAvoidance": '<Policy id="0" OptimizationMethod="gradient">'
                    '<costfunction range="5" name="FOEAvoidance" coeff="3"/>'
                    '<costfunction name="GoalReachingForce"/></Policy>',
}


def model_circle(model: str, n: int = 24, radius_m: float = 8.0, pref: float = 1.3, maxs: float = 1.6,
                 jitter: float = 0.01, seed: int = 10) -> Scenario:
    """n agents on a circle swapping sides, with one of the shipped model policies.

    Positions get a seeded jitter of +-``jitter`` m: on a perfectly symmetric
    circle many neighbour distances tie exactly, and the reference orders
    tied neighbours by its kd-tree traversal, which no other implementation
    reproduces (the summation order then differs in the last bit).
    """
    ang = 2.0 * np.pi * np.arange(n) / n
    pos = np.stack([radius_m * np.cos(ang), radius_m * np.sin(ang)], 1)
    if jitter:
        pos = pos + np.random.default_rng(seed).uniform(-jitter, jitter, pos.shape)
    return Scenario(dt=0.1, world="Infinite", policies=[MODEL_POLICIES[model]],
                    **_agents(n, pos, -pos, pref=pref, maxs=maxs))


def model_crossing(model: str, n: int = 40, seed: int = 11) -> Scenario:
    """Two jittered groups crossing at 90 degrees, with one of the model policies."""
    rng = np.random.default_rng(seed)
    h = n // 2
    a = np.stack([rng.uniform(-12, -6, h), rng.uniform(-3, 3, h)], 1)
    b = np.stack([rng.uniform(-3, 3, n - h), rng.uniform(-12, -6, n - h)], 1)
    pos = np.concatenate([a, b])
    goal = np.concatenate([a + [20, 0], b + [0, 20]])
    return Scenario(dt=0.1, world="Infinite", policies=[MODEL_POLICIES[model]],
                    **_agents(n, pos, goal, pref=1.3, maxs=1.6))


def model_arrivals(model: str, n: int = 40, seed: int = 17) -> Scenario:
    """Two crossing groups whose agents enter at staggered times (some at the
    same time) and leave at their goals (most of them): the dynamic
    population of WorldBase::DoStep (timed insertion, remove-at-goal)."""
    rng = np.random.default_rng(seed)
    h = n // 2
    a = np.stack([rng.uniform(-9, -5, h), rng.uniform(-2.5, 2.5, h)], 1)
    b = np.stack([rng.uniform(-2.5, 2.5, n - h), rng.uniform(-9, -5, n - h)], 1)
    pos = np.concatenate([a, b])
    goal = np.concatenate([a + [11, 0], b + [0, 11]])
    sc = Scenario(dt=0.1, world="Infinite", policies=[MODEL_POLICIES[model]],
                  **_agents(n, pos, goal, pref=1.3, maxs=1.6))
    start = np.round(rng.uniform(0.0, 4.0, n), 1).astype(np.float32)
    start[rng.random(n) < 0.3] = 0.0
    start[[1, 2, 3]] = start[0] = np.float32(1.5)      # a tie in the insertion queue
    sc.start_time = start
    sc.remove_at_goal = rng.random(n) < 0.8
    return sc


# Policies with the RandomFunction and Generic cost functions (the per-agent
# random stream consumed by sampling and by the costs themselves)
REGISTRY_POLICIES = {
    "RandomGradient": '<Policy id="0" OptimizationMethod="gradient" RelaxationTime="0.5">'
                      '<costfunction range="5" name="SocialForcesAvoidance"/>'
                      '<costfunction name="RandomFunction" coeff="0.5"/>'
                      '<costfunction name="GoalReachingForce"/></Policy>',
    "RandomSampling": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
                      'SamplingBaseDirection="unit" SamplingAngle="360" SpeedSamples="4" AngleSamples="36" '
                      'SamplingRadius="maximum speed" RelaxationTime="0.5">'
                      '<costfunction range="5" name="PowerLaw"/><costfunction name="RandomFunction" coeff="0.2"/>'
                      '<costfunction name="GoalReachingForce"/></Policy>',
    "RandomRVO": '<Policy id="0" OptimizationMethod="sampling" SamplingType="random" SamplingBase="current velocity" '
                 'SamplingBaseDirection="unit" SamplingAngle="360" RandomSamples="100" '
                 'SamplingRadius="maximum acceleration" RelaxationTime="0">'
                 '<costfunction range="5" name="RVO"/><costfunction name="RandomFunction" coeff="0.1"/></Policy>',
    "RandomGlobal": '<Policy id="0" OptimizationMethod="global" RelaxationTime="0.5">'
                    '<costfunction name="RandomFunction"/></Policy>',
    "GenericGlobal": '<Policy id="0" OptimizationMethod="global" RelaxationTime="0.5">'
                     '<costfunction name="Generic"/></Policy>',
    "GenericSampling": '<Policy id="0" OptimizationMethod="sampling" SamplingType="regular" SamplingBase="zero" '
                       'SamplingBaseDirection="preferred velocity" SamplingAngle="180" SpeedSamples="5" '
                       'AngleSamples="19" SamplingRadius="preferred speed" RelaxationTime="0.5">'
                       '<costfunction range="5" name="Moussaid"/><costfunction name="Generic"/></Policy>',
}


def registry_crossing(name: str, n: int = 40, seed: int = 16) -> Scenario:
    """The crossing layout with one of the RandomFunction / Generic policies."""
    sc = model_crossing("ORCA", n, seed)
    sc.policies = [REGISTRY_POLICIES[name]]
    return sc


BLOCK = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], np.float32)


def model_obstacle_crossing(model: str, n: int = 40, seed: int = 13) -> Scenario:
    """The crossing layout with a 2 x 2 m block at the crossing point."""
    sc = model_crossing(model, n, seed)
    sc.obstacles = [BLOCK.copy()]
    return sc


def model_corridor_walls(model: str, n: int = 40, seed: int = 14) -> Scenario:
    """Two groups walking in opposite directions along a 4 m wide corridor
    between two wall polygons (agents start close to the walls)."""
    rng = np.random.default_rng(seed)
    h = n // 2
    a = np.stack([rng.uniform(-10, -4, h), rng.uniform(-1.6, 1.6, h)], 1)
    b = np.stack([rng.uniform(4, 10, n - h), rng.uniform(-1.6, 1.6, n - h)], 1)
    pos = np.concatenate([a, b])
    goal = np.concatenate([a + [16, 0], b - [16, 0]])
    top = np.array([[-16, 2], [16, 2], [16, 2.5], [-16, 2.5]], np.float32)
    bottom = np.array([[-16, -2.5], [16, -2.5], [16, -2], [-16, -2]], np.float32)
    sc = Scenario(dt=0.1, world="Infinite", policies=[MODEL_POLICIES[model]],
                  **_agents(n, pos, goal, pref=1.3, maxs=1.6))
    sc.obstacles = [top, bottom]
    return sc


def model_toric_obstacle(model: str, n: int = 60, side: float = 8.0, seed: int = 15) -> Scenario:
    """The toric layout with a block next to the world's edge (displaced
    obstacle queries)."""
    sc = model_toric(model, n, side, seed)
    sc.obstacles = [BLOCK * 0.5 + np.array([side / 2 - 0.75, 0.0], np.float32)]
    return sc


def block_field(nblocks: int, side: float, rng, size=(0.3, 0.8), keep_clear=None) -> list:
    """nblocks small rotated quadrilaterals scattered in a side x side square
    (4 edges each), away from the points in keep_clear (k, 2)."""
    out = []
    while len(out) < nblocks:
        c = rng.uniform(-side / 2, side / 2, 2)
        if keep_clear is not None and len(keep_clear) and np.min(np.linalg.norm(keep_clear - c, axis=1)) < 1.2:
            continue
        h = rng.uniform(*size) / 2
        a = rng.uniform(0, np.pi / 2)
        rot = np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])
        sq = np.array([[-h, -h], [h, -h], [h, h], [-h, h]]) @ rot.T + c
        out.append(sq.astype(np.float32))
    return out


def model_block_field(model: str, n: int = 60, seed: int = 18) -> Scenario:
    """Agents crossing a 30 x 30 m field of 80 small blocks (320 edges: the
    edge-grid path of the obstacle query)."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-15, 15, (n, 2))
    goal = -pos + rng.uniform(-2, 2, (n, 2))
    sc = Scenario(dt=0.1, world="Infinite", policies=[MODEL_POLICIES[model]],
                  **_agents(n, pos, goal, pref=1.3, maxs=1.6))
    sc.obstacles = block_field(80, 30.0, rng, keep_clear=np.concatenate([pos, goal]))
    return sc


def model_toric_block_field(model: str, n: int = 60, side: float = 14.0, seed: int = 19) -> Scenario:
    """A 14 x 14 m toric world with 70 small blocks (280 edges), some next to
    the world's edges (displaced queries through the edge grid)."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-side / 2, side / 2, (n, 2))
    goal = pos + rng.uniform(-30, 30, (n, 2))
    sc = Scenario(dt=0.1, world="Toric", width=side, height=side, policies=[MODEL_POLICIES[model]],
                  **_agents(n, pos, goal, pref=1.3, maxs=1.6))
    sc.obstacles = block_field(70, side - 0.8, rng, size=(0.2, 0.5), keep_clear=pos)
    return sc


def model_toric(model: str, n: int = 60, side: float = 12.0, seed: int = 12) -> Scenario:
    """A small toric world (wrap-around neighbours, including displaced
    duplicates when the range exceeds half the side)."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-side / 2, side / 2, (n, 2))
    goal = pos + rng.uniform(-30, 30, (n, 2))
    return Scenario(dt=0.1, world="Toric", width=side, height=side, policies=[MODEL_POLICIES[model]],
                    **_agents(n, pos, goal, pref=1.3, maxs=1.6))
