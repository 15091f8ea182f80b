"""ctypes access to oracle/_ref/libumans_ref.so: the UMANS reference engine
compiled from its own sources (oracle/build_ref.sh) plus oracle/ref_shim.cpp.

Test infrastructure only.  The library exists only where the reference
sources were available to build it; ``available()`` says whether it does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libumans_ref.so")
_lib = None


def available() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    try:
        _load()
        return True
    except OSError:
        return False


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(LIB_PATH)
        lib.uref_load.restype = C.c_void_p
        lib.uref_load.argtypes = [C.c_char_p]
        lib.uref_free.argtypes = [C.c_void_p]
        lib.uref_num_agents.argtypes = [C.c_void_p]
        lib.uref_time.restype = C.c_double
        lib.uref_time.argtypes = [C.c_void_p]
        lib.uref_dt.restype = C.c_float
        lib.uref_dt.argtypes = [C.c_void_p]
        lib.uref_set_threads.argtypes = [C.c_void_p, C.c_int]
        lib.uref_step.restype = C.c_double
        lib.uref_step.argtypes = [C.c_void_p, C.c_int]
        P = C.c_void_p
        lib.uref_state.argtypes = [C.c_void_p, P, P, P, P, P, P]
        lib.uref_neighbors.argtypes = [C.c_void_p, C.c_int, P, P, P, P, C.c_int]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class RefSim:
    """One reference CrowdSimulator loaded from a scenario XML file."""

    def __init__(self, xml_path: str, threads: int = 1):
        lib = _load()
        self._h = lib.uref_load(os.fsencode(xml_path))
        if not self._h:
            raise RuntimeError(f"reference failed to load {xml_path}")
        lib.uref_set_threads(self._h, threads)

    def close(self):
        if self._h:
            _load().uref_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self) -> int:
        return _load().uref_num_agents(self._h)

    @property
    def time(self) -> float:
        return _load().uref_time(self._h)

    def step(self, n: int = 1) -> float:
        """Runs n steps; returns the seconds spent in RunSimulationSteps."""
        return _load().uref_step(self._h, n)

    def state(self) -> dict:
        n = self.n
        out = dict(ids=np.zeros(n, np.int64), pos=np.zeros((n, 2), np.float32),
                   vel=np.zeros((n, 2), np.float32), prefvel=np.zeros((n, 2), np.float32),
                   viewdir=np.zeros((n, 2), np.float32), goal=np.zeros((n, 2), np.float32))
        _load().uref_state(self._h, *(_p(out[k]) for k in ("ids", "pos", "vel", "prefvel", "viewdir", "goal")))
        return out

    def neighbors(self, idx: int, cap: int = 4096):
        """(ids, dist2, pos) of the list agent `idx` used in the last step."""
        ids = np.zeros(cap, np.int64)
        d2 = np.zeros(cap, np.float32)
        px = np.zeros(cap, np.float32)
        py = np.zeros(cap, np.float32)
        k = _load().uref_neighbors(self._h, idx, _p(ids), _p(d2), _p(px), _p(py), cap)
        k = min(k, cap)
        return ids[:k], d2[:k], np.stack([px[:k], py[:k]], 1)
