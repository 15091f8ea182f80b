"""ctypes access to the CPU restatement (oracle/port/umans_port.c), plus a
scenario reader that turns UMANS scenario XML into the port's flat arrays.

TEST INFRASTRUCTURE ONLY: tests, the golden-fixture tooling and bench.py's
CPU-baseline leg use this module; the product never imports it.

The XML reader follows the reference loader, src/Engine/core/crowdSimulator.cpp:
  * ``FromConfigFile`` (:516-647): ``configPath`` redirection, ``Simulation``
    ``delta_time``/``end_time``, ``World``, ``Policies``, ``Agents``;
  * ``...ExternallyOrNot`` (:210-274): a ``file=`` attribute loads the block
    from a file relative to the scenario's folder;
  * ``loadPoliciesBlock``/``loadAgentsBlock`` (:276-308): first child element,
    then following siblings with the block's element name;
  * ``loadSinglePolicy`` (:327-422): sampling attributes only for
    ``OptimizationMethod="sampling"``; cost functions are the first
    ``costfunction`` child and all following sibling elements; unknown names
    are skipped (``CostFunctionFactory::CreateCostFunction`` returns null);
  * ``loadSingleAgent`` (:424-494): agent defaults from ``Agent::Settings``
    (agent.h:44-53), ids assigned by ``WorldBase::AddAgent``
    (worldBase.cpp:161-186).
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import xml.etree.ElementTree as ET

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PORT_DIR = os.path.join(_HERE, "port")
LIB_PATH = os.path.join(PORT_DIR, "libumans_port.so")

KINDS = ["ORCA", "RVO", "SocialForcesAvoidance", "PowerLaw", "GoalReachingForce",
         "Karamouzas", "Moussaid", "Paris", "VanToll", "TtcaDca", "FOEAvoidance",
         "PLEdestrians", "RandomFunction", "Generic"]
# (attribute name, slot, default) per kind; defaults from the reference headers
PARAMS = {
    "ORCA": [("timeHorizon", 0, 5.0)],                                   # ORCA.h:54
    "RVO": [("w", 0, 1.0)],                                              # RVO.h:53
    "SocialForcesAvoidance": [("dt", 0, 1.0), ("V0", 1, 2.1), ("sigma", 2, 0.3),
                              ("U0", 1, None), ("R", 4, 0.2), ("agentMass", 5, 1.0)],
    "PowerLaw": [("k", 0, 1.5), ("tau0", 1, 3.0), ("agentMass", 5, 1.0)],  # PowerLaw.h:57-58
    "GoalReachingForce": [("agentMass", 5, 1.0)],
    "Karamouzas": [("alpha", 0, 5.0), ("beta", 1, 0.5), ("gamma", 2, 1.0),
                   ("delta", 3, 1.0), ("t_max", 4, 8.0)],                # Karamouzas.h:49-53
    "Moussaid": [("d_max", 0, 8.0)],
    "Paris": [("w_a", 0, 0.5), ("w_b", 1, 0.0), ("t_max", 2, 8.0)],
    "VanToll": [("max_distance", 0, 8.0)],
    "TtcaDca": [("sigmaAngle_goal", 0, 2.0), ("sigmaSpeed_goal", 1, 2.0),
                ("sigmaTtca", 2, 1.0), ("sigmaDca", 3, 0.3)],
    "FOEAvoidance": [],
    "PLEdestrians": [("w_a", 0, 2.23), ("w_b", 1, 1.26), ("t_min", 2, 0.5), ("t_max", 3, 3.0)],
    "RandomFunction": [],
    "Generic": [],
}
# the U0 attribute is read into V0 (SocialForcesAvoidance.cpp:148); U0 itself
# keeps its default 10 in slot 3 and is only used by obstacle forces.
DEFAULT_RANGE = {"GoalReachingForce": 0.0, "RandomFunction": 0.0}   # RandomFunction.h: range_ = 0


class CostT(C.Structure):
    _fields_ = [("kind", C.c_int), ("coeff", C.c_float), ("range", C.c_float),
                ("p", C.c_float * 8)]


class PolicyT(C.Structure):
    _fields_ = [("method", C.c_int), ("s_type", C.c_int), ("s_base", C.c_int),
                ("s_dir", C.c_int), ("s_radius", C.c_int), ("s_angle", C.c_float),
                ("speed_samples", C.c_int), ("angle_samples", C.c_int),
                ("random_samples", C.c_int), ("include_base", C.c_int),
                ("relax_time", C.c_float), ("contact_scale", C.c_float),
                ("ncost", C.c_int), ("cost", CostT * 8)]


def _f32(s: str) -> float:
    return float(np.float32(float(s.strip())))


def _int(s: str):
    try:
        return int(s.strip(), 0)
    except ValueError:
        return None


def _bool(s: str):
    v = _int(s)
    if v is not None:
        return v != 0
    t = s.strip()
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    return None


def _children_from_first(block, name):
    kids = list(block)
    if not kids:
        return []
    out = [kids[0]]
    out += [k for k in kids[1:] if k.tag == name]
    return out


def _parse_lenient(path: str):
    """Parses a file the way tinyxml2 accepts it: several top-level elements
    and comments containing '--' are allowed.  Returns a synthetic root whose
    children are the document's top-level elements."""
    with open(path, "rb") as fh:
        text = fh.read().decode("utf-8", errors="replace")
    text = re.sub(r"<!--.*?-->", "", text, flags=re.S)
    text = re.sub(r"<\?.*?\?>", "", text, flags=re.S)
    return ET.fromstring("<document>" + text + "</document>")


def _load_block(elem, folder, name):
    f = elem.get("file")
    if f is not None:
        root = _parse_lenient(os.path.join(folder, f)).find(name)
        if root is None:
            raise ValueError(f"could not load {name} from {f}")
        return root
    return elem


def read_scenario(path: str) -> dict:
    """Parses a scenario file into the arrays ``PortSim`` takes."""
    folder = os.path.dirname(path)
    doc = _parse_lenient(path)
    cfg = doc.find("configPath")
    if cfg is not None:
        return read_scenario(os.path.join(folder, cfg.get("path")))
    sim = doc.find("Simulation")
    if sim is None:
        raise ValueError("no Simulation element")
    world = sim.find("World")
    wtype = world.get("type", "Infinite")
    width = height = 0.0
    toric = wtype == "Toric"
    if toric:
        width, height = _f32(world.get("width", "-1")), _f32(world.get("height", "-1"))
        if not (width > 0 and height > 0):
            raise ValueError("invalid toric size")
    dt = _f32(sim.get("delta_time", "-1"))
    if not dt > 0:
        raise ValueError("invalid delta_time")
    end_time = _f32(sim.get("end_time")) if sim.get("end_time") else None

    policies, policy_ids = [], []
    pblock = sim.find("Policies")
    if pblock is not None:
        pblock = _load_block(pblock, folder, "Policies")
        for pe in _children_from_first(pblock, "Policy"):
            pid = _int(pe.get("id", "0"))
            method = {"gradient": 0, "sampling": 1, "global": 2}.get(pe.get("OptimizationMethod", ""))
            if method is None:
                raise ValueError(f"policy {pid}: invalid optimization method")
            P = PolicyT()
            P.method = method
            P.s_type, P.s_base, P.s_dir, P.s_radius = 0, 0, 1, 0   # policy.h:59-67 defaults
            P.s_angle, P.speed_samples, P.angle_samples, P.random_samples, P.include_base = 180.0, 4, 11, 100, 0
            if method == 1:
                if pe.get("SamplingAngle") is not None:
                    P.s_angle = _f32(pe.get("SamplingAngle"))
                for a, fld in (("SpeedSamples", "speed_samples"), ("AngleSamples", "angle_samples"),
                               ("RandomSamples", "random_samples")):
                    if pe.get(a) is not None and _int(pe.get(a)) is not None:
                        setattr(P, fld, _int(pe.get(a)))
                if pe.get("IncludeBaseAsSample") is not None and _bool(pe.get("IncludeBaseAsSample")) is not None:
                    P.include_base = int(_bool(pe.get("IncludeBaseAsSample")))
                P.s_type = {"regular": 0, "random": 1}.get(pe.get("SamplingType", "regular"), P.s_type)
                P.s_base = {"zero": 0, "current velocity": 1}.get(pe.get("SamplingBase", "zero"), P.s_base)
                P.s_dir = {"unit": 0, "current velocity": 1, "preferred velocity": 2}.get(
                    pe.get("SamplingBaseDirection", "current velocity"), P.s_dir)
                P.s_radius = {"preferred speed": 0, "maximum speed": 1, "maximum acceleration": 2}.get(
                    pe.get("SamplingRadius", "preferred speed"), P.s_radius)
            P.relax_time = _f32(pe.get("RelaxationTime")) if pe.get("RelaxationTime") is not None else 0.0
            P.contact_scale = _f32(pe.get("ContactForceScale")) if pe.get("ContactForceScale") is not None else 5000.0
            kids = list(pe)
            first = next((i for i, k in enumerate(kids) if k.tag == "costfunction"), None)
            n = 0
            if first is not None:
                for ce in kids[first:]:
                    name = ce.get("name")
                    if name not in KINDS:
                        continue
                    c = P.cost[n]
                    c.kind = KINDS.index(name)
                    c.coeff = _f32(ce.get("coeff")) if ce.get("coeff") is not None else 1.0
                    c.range = DEFAULT_RANGE.get(name, 5.0)
                    if ce.get("range") is not None:
                        c.range = _f32(ce.get("range"))
                    vals = [0.0] * 8
                    for attr, slot, dflt in PARAMS[name]:
                        if dflt is not None:
                            vals[slot] = dflt
                    if name == "SocialForcesAvoidance":
                        vals[3] = 10.0
                    for attr, slot, dflt in PARAMS[name]:
                        if ce.get(attr) is not None:
                            vals[slot] = _f32(ce.get(attr))
                    for k in range(8):
                        c.p[k] = vals[k]
                    n += 1
            if n == 0:
                raise ValueError(f"policy {pid} needs at least one cost function")
            P.ncost = n
            if pid in policy_ids:
                raise ValueError(f"policy id {pid} taken")
            policies.append(P)
            policy_ids.append(pid)
    if not policies:
        raise ValueError("no policies")

    ids, pos, goal, rad, pref, maxs, maxa, pidx = [], [], [], [], [], [], [], []
    start, rmg = [], []
    taken = set()
    next_id = 0
    ablock = sim.find("Agents")
    if ablock is not None:
        ablock = _load_block(ablock, folder, "Agents")
        for ae in _children_from_first(ablock, "Agent"):
            want = _int(ae.get("id")) if ae.get("id") is not None else -1
            r = _f32(ae.get("rad")) if ae.get("rad") is not None else float(np.float32(0.24))
            ps = _f32(ae.get("pref_speed")) if ae.get("pref_speed") is not None else float(np.float32(1.4))
            ms = _f32(ae.get("max_speed")) if ae.get("max_speed") is not None else float(np.float32(1.8))
            ma = _f32(ae.get("max_acceleration")) if ae.get("max_acceleration") is not None else 5.0
            pe = ae.find("pos")
            if pe is None:
                raise ValueError("agent needs a position")
            p = (_f32(pe.get("x")), _f32(pe.get("y")))
            pol = ae.find("Policy")
            if pol is None or _int(pol.get("id")) not in policy_ids:
                raise ValueError("agent policy missing")
            if want is not None and want >= 0 and want not in taken:
                aid = want
            else:
                aid = next_id
            if aid >= next_id:
                next_id = aid + 1
            taken.add(aid)
            ge = ae.find("goal")
            g = (_f32(ge.get("x")), _f32(ge.get("y"))) if ge is not None else p
            ids.append(aid); pos.append(p); goal.append(g); rad.append(r); pref.append(ps)
            maxs.append(ms); maxa.append(ma); pidx.append(policy_ids.index(_int(pol.get("id"))))
            # crowdSimulator.cpp:436, 470-475 (QueryBoolAttribute / QueryFloatAttribute)
            st = _f32(ae.get("start_time")) if ae.get("start_time") is not None else 0.0
            rg = _bool(ae.get("remove_at_goal")) if ae.get("remove_at_goal") is not None else False
            start.append(st)
            rmg.append(bool(rg))
    # obstacles (crowdSimulator.cpp:496-514, 633-645): every polygon's
    # closed outline, polygons in file order (Polygon2D.cpp:27-35)
    edges = []
    oblock = world.find("Obstacles")
    if oblock is not None:
        oblock = _load_block(oblock, folder, "Obstacles")
        for oe in _children_from_first(oblock, "Obstacle"):
            pts = [(_f32(pe.get("x", "0")), _f32(pe.get("y", "0"))) for pe in oe.findall("Point")]
            for k in range(len(pts)):
                a, b = pts[k], pts[(k + 1) % len(pts)]
                edges.append((a[0], a[1], b[0], b[1]))
    f = np.float32
    return dict(world=1 if toric else 0, width=width, height=height, dt=dt, end_time=end_time,
                edges=np.array(edges, f).reshape(-1, 4),
                policies=policies, ids=np.array(ids, np.int64),
                pos=np.array(pos, f).reshape(-1, 2), goal=np.array(goal, f).reshape(-1, 2),
                radius=np.array(rad, f), pref_speed=np.array(pref, f), max_speed=np.array(maxs, f),
                max_accel=np.array(maxa, f), policy_index=np.array(pidx, np.int32),
                start_time=np.array(start, f), remove_at_goal=np.array(rmg, np.uint8))


_lib = None


def build(force: bool = False) -> str:
    """Compiles the port (gcc, -ffp-contract=off) into oracle/port/libumans_port.so."""
    src = os.path.join(PORT_DIR, "umans_port.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(src) > os.path.getmtime(LIB_PATH):
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-fPIC",
                               "-shared", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


def _load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        lib.up_create.restype = C.c_void_p
        lib.up_create.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, P, C.c_int,
                                  P, P, P, P, P, P, P, P]
        lib.up_free.argtypes = [P]
        lib.up_num_agents.argtypes = [P]
        lib.up_time.restype = C.c_double
        lib.up_time.argtypes = [P]
        lib.up_step.restype = C.c_double
        lib.up_step.argtypes = [P, C.c_int, C.c_int]
        lib.up_state.argtypes = [P, P, P, P, P, P, P]
        lib.up_set_state.argtypes = [P, P, P, P]
        lib.up_neighbors.argtypes = [P, C.c_int, P, P, P, P, C.c_int]
        lib.up_libm_expf.argtypes = [P, P, C.c_long]
        lib.up_libm_sincosf.argtypes = [P, P, P, C.c_long]
        lib.up_set_dynamics.argtypes = [P, P, P]
        lib.up_set_obstacles.argtypes = [P, C.c_int, P]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def libm_expf(x: np.ndarray) -> np.ndarray:
    """The host C library's expf, elementwise (float32)."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    _load().up_libm_expf(_p(x), _p(y), x.size)
    return y


def libm_sincosf(x: np.ndarray):
    """The host C library's sinf and cosf, elementwise (float32)."""
    x = np.ascontiguousarray(x, np.float32)
    s, c = np.empty_like(x), np.empty_like(x)
    _load().up_libm_sincosf(_p(x), _p(s), _p(c), x.size)
    return s, c


class PortSim:
    """The CPU restatement loaded from a scenario file (or a parsed dict)."""

    def __init__(self, scenario, threads: int = 1):
        lib = _load()
        s = read_scenario(scenario) if isinstance(scenario, str) else scenario
        self.s = s
        self.threads = threads
        pols = (PolicyT * len(s["policies"]))(*s["policies"])
        self._keep = [np.ascontiguousarray(s[k]) for k in
                      ("ids", "pos", "goal", "radius", "pref_speed", "max_speed", "max_accel", "policy_index")]
        self._h = lib.up_create(len(s["ids"]), s["world"], s["width"], s["height"], s["dt"],
                                C.cast(pols, C.c_void_p), len(s["policies"]), *(_p(a) for a in self._keep))
        st = np.ascontiguousarray(s.get("start_time", np.zeros(0, np.float32)), np.float32)
        rg = np.ascontiguousarray(s.get("remove_at_goal", np.zeros(0, np.uint8)), np.uint8)
        if (st.size and (st > 0).any()) or (rg.size and rg.any()):
            self._keep += [st, rg]
            lib.up_set_dynamics(self._h, _p(st), _p(rg))
        edges = np.ascontiguousarray(s.get("edges", np.zeros((0, 4), np.float32)), np.float32)
        if edges.shape[0]:
            self._keep.append(edges)
            lib.up_set_obstacles(self._h, edges.shape[0], _p(edges))

    def close(self):
        if self._h:
            _load().up_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self) -> int:
        return _load().up_num_agents(self._h)

    @property
    def time(self) -> float:
        return _load().up_time(self._h)

    def step(self, n: int = 1) -> float:
        return _load().up_step(self._h, n, self.threads)

    def state(self) -> dict:
        n = self.n
        out = dict(ids=np.zeros(n, np.int64), pos=np.zeros((n, 2), np.float32),
                   vel=np.zeros((n, 2), np.float32), prefvel=np.zeros((n, 2), np.float32),
                   viewdir=np.zeros((n, 2), np.float32), goal=np.zeros((n, 2), np.float32))
        _load().up_state(self._h, *(_p(out[k]) for k in ("ids", "pos", "vel", "prefvel", "viewdir", "goal")))
        return out

    def set_state(self, pos=None, vel=None, viewdir=None):
        a = [None if x is None else np.ascontiguousarray(x, np.float32) for x in (pos, vel, viewdir)]
        _load().up_set_state(self._h, *(_p(x) for x in a))

    def neighbors(self, idx: int, cap: int = 8192):
        ids = np.zeros(cap, np.int64)
        d2 = np.zeros(cap, np.float32)
        px = np.zeros(cap, np.float32)
        py = np.zeros(cap, np.float32)
        k = min(_load().up_neighbors(self._h, idx, _p(ids), _p(d2), _p(px), _p(py), cap), cap)
        return ids[:k], d2[:k], np.stack([px[:k], py[:k]], 1)
