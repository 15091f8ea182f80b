"""Python-facing classes over the C ABI."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import AgentData


class UmansError(RuntimeError):
    pass


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Simulation:
    """One simulation on the GPU (the reference's CrowdSimulator + World).

    ``Simulation(path)`` loads a UMANS scenario file with the reference's
    loader semantics (CrowdSimulator::FromConfigFile).
    """

    def __init__(self, config_file: str, max_neighbours: int = 0, cells_per_range: float = 0.0,
                 use_graph: bool = True):
        lib = _lib.load()
        h = C.c_void_p()
        rc = lib.umans_create_ex(os.fsencode(config_file), int(max_neighbours), float(cells_per_range),
                                 int(bool(use_graph)), C.byref(h))
        if rc != 0:
            raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
        self._lib = lib
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise UmansError(self._lib.umans_last_error(self._h).decode(errors="replace"))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.umans_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- stepping -------------------------------------------------------
    def step(self, n: int = 1):
        self._check(self._lib.umans_step(self._h, int(n)))

    def step_async(self, n: int = 1):
        self._check(self._lib.umans_step_async(self._h, int(n)))

    def synchronize(self):
        self._check(self._lib.umans_synchronize(self._h))

    # --- properties -----------------------------------------------------
    @property
    def n(self) -> int:
        v = C.c_int()
        self._check(self._lib.umans_num_agents(self._h, C.byref(v)))
        return v.value

    @property
    def time(self) -> float:
        v = C.c_double()
        self._check(self._lib.umans_time(self._h, C.byref(v)))
        return v.value

    @property
    def dt(self) -> float:
        v = C.c_float()
        self._check(self._lib.umans_dt(self._h, C.byref(v)))
        return v.value

    @property
    def end_time(self) -> float:
        v = C.c_float()
        self._check(self._lib.umans_end_time(self._h, C.byref(v)))
        return v.value

    @property
    def max_neighbours(self) -> int:
        v = C.c_int()
        self._check(self._lib.umans_max_neighbours(self._h, C.byref(v)))
        return v.value

    @property
    def stream(self) -> int:
        v = C.c_void_p()
        self._check(self._lib.umans_stream(self._h, C.byref(v)))
        return v.value or 0

    def device_state(self):
        p, v = C.c_void_p(), C.c_void_p()
        self._check(self._lib.umans_device_state(self._h, C.byref(p), C.byref(v)))
        return p.value, v.value

    def autotune(self, trial_steps: int = 3) -> dict:
        cpr, occ = C.c_float(), C.c_float()
        wpb, sched, lanes = C.c_int(), C.c_int(), C.c_int()
        self._check(self._lib.umans_autotune(self._h, int(trial_steps), C.byref(cpr), C.byref(wpb), C.byref(occ),
                                             C.byref(sched), C.byref(lanes)))
        return dict(cells_per_range=cpr.value, warps_per_block=wpb.value, occupancy=occ.value, schedule=sched.value,
                    agent_lanes=lanes.value)

    def set_launch(self, cells_per_range: float = 2.0, warps_per_block: int = 4, occupancy: float = 1.0,
                   schedule: int = 0, agent_lanes: int = 8):
        """Applies a launch shape (as autotune reports one); results do not depend on it."""
        self._check(self._lib.umans_set_launch(self._h, float(cells_per_range), int(warps_per_block),
                                               float(occupancy), int(schedule), int(agent_lanes)))

    def set_multi_step(self, enable: bool = True):
        """Small worlds: the steps of one call in one launch (the default), or
        one graph launch per step; results do not depend on it."""
        self._check(self._lib.umans_set_multi_step(self._h, int(bool(enable))))

    def profile(self, enable: bool = True):
        self._check(self._lib.umans_profile(self._h, int(bool(enable))))

    def profile_totals(self) -> dict:
        a, b, g = C.c_double(), C.c_double(), C.c_double()
        n, k = C.c_int(), C.c_int()
        self._check(self._lib.umans_profile_totals(self._h, C.byref(a), C.byref(b), C.byref(n), C.byref(k),
                                                   C.byref(g)))
        return dict(agent_kernel_ms=a.value, step_ms=b.value, steps=n.value, kernels_per_step=k.value,
                    grid_build_ms=g.value)

    def profile_counters(self) -> dict:
        c = np.zeros(3, np.uint64)
        self._check(self._lib.umans_profile_counters(self._h, _p(c), 3))
        return dict(karamouzas_window_samples=int(c[0]), karamouzas_pair_ttc=int(c[1]),
                    karamouzas_agents=int(c[2]))

    # --- state ----------------------------------------------------------
    def state(self) -> dict:
        n = self.n
        out = dict(ids=np.zeros(n, np.int32), pos=np.zeros((n, 2), np.float32),
                   vel=np.zeros((n, 2), np.float32), viewdir=np.zeros((n, 2), np.float32))
        self._check(self._lib.umans_get_state(self._h, _p(out["ids"]), _p(out["pos"]), _p(out["vel"]),
                                              _p(out["viewdir"]), n))
        pv = np.zeros((n, 2), np.float32)
        g = np.zeros((n, 2), np.float32)
        self._check(self._lib.umans_get_aux(self._h, _p(pv), _p(g), n))
        out["prefvel"] = pv
        out["goal"] = g
        return out

    def positions(self) -> np.ndarray:
        n = self.n
        pos = np.zeros((n, 2), np.float32)
        self._check(self._lib.umans_get_state(self._h, None, _p(pos), None, None, n))
        return pos

    def set_state(self, pos=None, vel=None, viewdir=None):
        a = [None if x is None else np.ascontiguousarray(x, np.float32) for x in (pos, vel, viewdir)]
        for x in a:
            if x is not None and x.size != 2 * self.n:
                raise ValueError("state arrays must have shape (n, 2)")
        self._check(self._lib.umans_set_state(self._h, *(_p(x) for x in a)))

    def get_agents(self, out=None):
        """GetAgentPositions into a ctypes AgentData array (reused if given)."""
        n = self.n
        if out is None or len(out) < n:
            out = (AgentData * max(n, 1))()
        cnt = C.c_int()
        self._check(self._lib.umans_get_agents(self._h, out, len(out), C.byref(cnt)))
        return out, cnt.value

    def set_agents(self, agents):
        arr = (AgentData * len(agents))(*agents)
        self._check(self._lib.umans_set_agents(self._h, arr, len(agents)))

    def add_agent(self, x, y, radius, pref_speed, max_speed, max_acceleration, policy_id, desired_id=-1) -> int:
        out = C.c_int()
        self._check(self._lib.umans_add_agent(self._h, x, y, radius, pref_speed, max_speed, max_acceleration,
                                              int(policy_id), int(desired_id), C.byref(out)))
        return out.value

    def remove_agent(self, agent_id: int):
        self._check(self._lib.umans_remove_agent(self._h, int(agent_id)))

    def set_goal(self, agent_id: int, x: float, y: float):
        self._check(self._lib.umans_set_goal(self._h, int(agent_id), float(x), float(y)))

    def neighbours(self, cap: int = 64):
        """(ids[n, cap], dist2[n, cap], counts[n]) of the lists the next step uses."""
        n = self.n
        ids = np.full((n, cap), -1, np.int32)
        d2 = np.zeros((n, cap), np.float32)
        cnt = np.zeros(n, np.int32)
        self._check(self._lib.umans_neighbours(self._h, int(cap), _p(ids), _p(d2), _p(cnt)))
        return ids, d2, cnt

    # --- trajectory output ------------------------------------------------
    def record_start(self, directory: str, ring_steps: int = 64, binary: bool = False):
        """Write every step's positions to `directory`: output_<id>.csv per
        agent (the reference's CSVWriter layout, full float precision), or
        trajectory.bin with `binary` (read it with read_trajectory)."""
        self._check(self._lib.umans_record_start(self._h, os.fsencode(directory), int(ring_steps), int(bool(binary))))

    def record_flush(self):
        self._check(self._lib.umans_record_flush(self._h))

    def record_stop(self):
        self._check(self._lib.umans_record_stop(self._h))

    @property
    def num_scenarios(self) -> int:
        ns = C.c_int()
        self._check(self._lib.umans_batch_offsets(self._h, None, 0, C.byref(ns)))
        return ns.value

    # --- differentiable form (calibration) ------------------------------
    def set_force_params(self, params, scenario: int = -1):
        """(V0, sigma, k, tau0) of the SocialForcesAvoidance / PowerLaw costs
        of one scenario (all when scenario < 0); NaN entries stay unchanged."""
        a = np.ascontiguousarray(params, np.float32).reshape(4)
        self._check(self._lib.umans_set_force_params(self._h, int(scenario), _p(a)))

    def force_params(self, scenario: int = 0) -> np.ndarray:
        a = np.zeros(4, np.float32)
        self._check(self._lib.umans_get_force_params(self._h, int(scenario), _p(a)))
        return a

    def diff_begin(self, targets, checkpoint_every: int = 10, weight: float = 0.0):
        """Start an episode from the current state: targets[t, i] is the
        position agent i should have after step t + 1 (list order)."""
        t = np.ascontiguousarray(targets, np.float32)
        if t.ndim != 3 or t.shape[1:] != (self.n, 2):
            raise ValueError("targets must have shape (steps, n, 2)")
        self._check(self._lib.umans_diff_begin(self._h, t.shape[0], int(checkpoint_every), _p(t), float(weight)))
        self._diff_steps = t.shape[0]

    def diff_forward(self) -> float:
        loss = C.c_double()
        self._check(self._lib.umans_diff_forward(self._h, C.byref(loss)))
        return loss.value

    def diff_backward(self, with_state: bool = False):
        """dL/d(V0, sigma, k, tau0) per scenario [num_scenarios, 4]; with
        with_state also dL/d(initial positions) and dL/d(initial velocities)."""
        dp = np.zeros((self.num_scenarios, 4), np.float32)
        if not with_state:
            self._check(self._lib.umans_diff_backward(self._h, _p(dp), None, None))
            return dp
        gp = np.zeros((self.n, 2), np.float32)
        gv = np.zeros((self.n, 2), np.float32)
        self._check(self._lib.umans_diff_backward(self._h, _p(dp), _p(gp), _p(gv)))
        return dp, gp, gv

    def diff_end(self):
        self._check(self._lib.umans_diff_end(self._h))


def scenario_info(config_file: str) -> dict:
    """Loads a scenario file on the host only: agents (timed insertions
    included), policies and obstacle edges.  Raises UmansError with the
    loader's message when the file would not load."""
    lib = _lib.load()
    a, p, e = C.c_int(), C.c_int(), C.c_int()
    if lib.umans_scenario_info(os.fsencode(config_file), C.byref(a), C.byref(p), C.byref(e)) != 0:
        raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
    return dict(agents=a.value, policies=p.value, edges=e.value)


def scenario_warnings(config_file: str) -> list:
    """The loader's warnings for a scenario file (host only): what the
    reference reports on standard error while loading it."""
    lib = _lib.load()
    need = C.c_int()
    path = os.fsencode(config_file)
    if lib.umans_scenario_warnings(path, None, 0, C.byref(need)) != 0:
        raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
    buf = C.create_string_buffer(need.value)
    if lib.umans_scenario_warnings(path, buf, need.value, C.byref(need)) != 0:
        raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
    return [w for w in buf.value.decode(errors="replace").split("\n") if w]


def cost_functions() -> list:
    """Names a policy's cost functions may use: the built-in costs, then the
    compiled-in plugins (the reference's CostFunctionFactory registry)."""
    lib = _lib.load()
    n = C.c_int()
    if lib.umans_cost_functions(None, 0, C.byref(n)) != 0:
        raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
    buf = (C.c_char_p * n.value)()
    if lib.umans_cost_functions(buf, n.value, C.byref(n)) != 0:
        raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
    return [b.decode() for b in buf]


def read_trajectory(path: str):
    """Chunks of a trajectory.bin written by Simulation.record_start(binary=True):
    a list of (ids[n], times[steps], xy[steps, n, 2])."""
    import struct
    out = []
    with open(path, "rb") as fh:
        data = fh.read()
    off = 0
    while off < len(data):
        if data[off:off + 4] != b"UMTR":
            raise ValueError("not a trajectory chunk at byte %d" % off)
        n, steps = struct.unpack_from("<ii", data, off + 4)
        off += 12
        ids = np.frombuffer(data, np.int32, n, off).copy()
        off += 4 * n
        times = np.frombuffer(data, np.float64, steps, off).copy()
        off += 8 * steps
        xy = np.frombuffer(data, np.float32, steps * n * 2, off).reshape(steps, n, 2).copy()
        off += 4 * steps * n * 2
        out.append((ids, times, xy))
    return out


class Batch(Simulation):
    """Several independent scenarios stepped together on the GPU.

    ``Batch(paths)``: agents of scenario k are at list slots
    ``offsets[k]:offsets[k+1]`` of every state array.  Each scenario evolves
    exactly as a ``Simulation`` of its own file.
    """

    def __init__(self, config_files):
        lib = _lib.load()
        arr = (C.c_char_p * len(config_files))(*[os.fsencode(f) for f in config_files])
        h = C.c_void_p()
        rc = lib.umans_batch_create(arr, len(config_files), C.byref(h))
        if rc != 0:
            raise UmansError(lib.umans_last_error(None).decode(errors="replace"))
        self._lib = lib
        self._h = h

    @property
    def offsets(self) -> np.ndarray:
        ns = C.c_int()
        self._check(self._lib.umans_batch_offsets(self._h, None, 0, C.byref(ns)))
        off = np.zeros(ns.value + 1, np.int32)
        self._check(self._lib.umans_batch_offsets(self._h, _p(off), off.size, None))
        return off

    def autotune(self, trial_steps: int = 3) -> dict:
        cpr, occ = C.c_float(), C.c_float()
        wpb, sched, lanes = C.c_int(), C.c_int(), C.c_int()
        self._check(self._lib.umans_autotune(self._h, int(trial_steps), C.byref(cpr), C.byref(wpb), C.byref(occ),
                                             C.byref(sched), C.byref(lanes)))
        return dict(cells_per_range=cpr.value, warps_per_block=wpb.value, occupancy=occ.value, schedule=sched.value,
                    agent_lanes=lanes.value)

    def set_launch(self, cells_per_range: float = 2.0, warps_per_block: int = 4, occupancy: float = 1.0,
                   schedule: int = 0, agent_lanes: int = 8):
        """Applies a launch shape (as autotune reports one); results do not depend on it."""
        self._check(self._lib.umans_set_launch(self._h, float(cells_per_range), int(warps_per_block),
                                               float(occupancy), int(schedule), int(agent_lanes)))


class UMANS:
    """The reference's Python interface (src/Library/PyAPI.h:55-246) on the
    reference-compatible global C functions."""

    def __init__(self):
        self._lib = _lib.load()

    def startSimulation(self, configFileName: str, numberOfThreads: int = 1) -> bool:
        return bool(self._lib.StartSimulation(os.fsencode(configFileName), int(numberOfThreads)))

    def getSimulationTimeStep(self) -> float:
        v = C.c_float(-1)
        if not self._lib.GetSimulationTimeStep(C.byref(v)):
            return -1.0
        return v.value

    def doSimulationSteps(self, nrSteps: int) -> bool:
        return bool(self._lib.DoSimulationSteps(int(nrSteps)))

    def getAgentPositions(self) -> list:
        ptr = C.POINTER(AgentData)()
        n = C.c_int()
        if not self._lib.GetAgentPositions(C.byref(ptr), C.byref(n)):
            return []
        out = []
        for i in range(n.value):
            a = ptr[i]
            out.append(AgentData(a.id, a.position_x, a.position_y, a.velocity_x, a.velocity_y,
                                 a.viewingDirection_x, a.viewingDirection_y))
        return out

    def setAgentPositions(self, agentData) -> bool:
        arr = (AgentData * len(agentData))(*agentData)
        return bool(self._lib.SetAgentPositions(arr, len(agentData)))

    def addAgent(self, x, y, radius, prefSpeed, maxSpeed, maxAcceleration, policyID, customID=-1) -> int:
        out = C.c_int(-1)
        ok = self._lib.AddAgent(x, y, radius, prefSpeed, maxSpeed, maxAcceleration, int(policyID),
                                C.byref(out), int(customID))
        return out.value if ok else -1

    def removeAgent(self, id: int) -> bool:
        return bool(self._lib.RemoveAgent(int(id)))

    def setAgentGoal(self, id: int, x: float, y: float) -> bool:
        return bool(self._lib.SetAgentGoal(int(id), float(x), float(y)))

    def cleanUp(self) -> bool:
        return bool(self._lib.CleanUp())

    def getNumberOfAgents(self) -> int:
        return len(self.getAgentPositions())

    def getNumberOfObstacles(self) -> int:
        return 0
