"""Loads libumans_gb300.so and declares the C ABI of include/umans_gb300.h.

The library is built in-tree (umans_gb300/build.py).  There is no CPU
fallback: if the library is missing, or no CUDA device is present when a
simulation is created, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libumans_gb300.so")


class AgentData(C.Structure):
    """struct AgentData (reference src/Library/APIFunctions.h:33-49)."""
    _fields_ = [("id", C.c_int), ("position_x", C.c_float), ("position_y", C.c_float),
                ("velocity_x", C.c_float), ("velocity_y", C.c_float),
                ("viewingDirection_x", C.c_float), ("viewingDirection_y", C.c_float)]


# name -> (restype, argtypes)
P = C.c_void_p
_SIGS = {
    "StartSimulation": (C.c_bool, [C.c_char_p, C.c_int]),
    "GetSimulationTimeStep": (C.c_bool, [C.POINTER(C.c_float)]),
    "DoSimulationSteps": (C.c_bool, [C.c_int]),
    "GetAgentPositions": (C.c_bool, [C.POINTER(C.POINTER(AgentData)), C.POINTER(C.c_int)]),
    "SetAgentPositions": (C.c_bool, [C.POINTER(AgentData), C.c_int]),
    "AddAgent": (C.c_bool, [C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                            C.POINTER(C.c_int), C.c_int]),
    "RemoveAgent": (C.c_bool, [C.c_int]),
    "SetAgentGoal": (C.c_bool, [C.c_int, C.c_float, C.c_float]),
    "CleanUp": (C.c_bool, []),
    "umans_create": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "umans_create_ex": (C.c_int, [C.c_char_p, C.c_int, C.c_float, C.c_int, C.POINTER(P)]),
    "umans_destroy": (C.c_int, [P]),
    "umans_batch_create": (C.c_int, [C.POINTER(C.c_char_p), C.c_int, C.POINTER(P)]),
    "umans_batch_offsets": (C.c_int, [P, P, C.c_int, C.POINTER(C.c_int)]),
    "umans_autotune": (C.c_int, [P, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_float),
                                 C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "umans_set_launch": (C.c_int, [P, C.c_float, C.c_int, C.c_float, C.c_int, C.c_int]),
    "umans_set_multi_step": (C.c_int, [P, C.c_int]),
    "umans_step": (C.c_int, [P, C.c_int]),
    "umans_step_async": (C.c_int, [P, C.c_int]),
    "umans_synchronize": (C.c_int, [P]),
    "umans_num_agents": (C.c_int, [P, C.POINTER(C.c_int)]),
    "umans_time": (C.c_int, [P, C.POINTER(C.c_double)]),
    "umans_dt": (C.c_int, [P, C.POINTER(C.c_float)]),
    "umans_end_time": (C.c_int, [P, C.POINTER(C.c_float)]),
    "umans_get_state": (C.c_int, [P, P, P, P, P, C.c_int]),
    "umans_get_aux": (C.c_int, [P, P, P, C.c_int]),
    "umans_set_state": (C.c_int, [P, P, P, P]),
    "umans_set_agents": (C.c_int, [P, C.POINTER(AgentData), C.c_int]),
    "umans_get_agents": (C.c_int, [P, C.POINTER(AgentData), C.c_int, C.POINTER(C.c_int)]),
    "umans_add_agent": (C.c_int, [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                  C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "umans_remove_agent": (C.c_int, [P, C.c_int]),
    "umans_set_goal": (C.c_int, [P, C.c_int, C.c_float, C.c_float]),
    "umans_neighbours": (C.c_int, [P, C.c_int, P, P, P]),
    "umans_max_neighbours": (C.c_int, [P, C.POINTER(C.c_int)]),
    "umans_stream": (C.c_int, [P, C.POINTER(P)]),
    "umans_device_state": (C.c_int, [P, C.POINTER(P), C.POINTER(P)]),
    "umans_profile": (C.c_int, [P, C.c_int]),
    "umans_profile_totals": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "umans_profile_counters": (C.c_int, [P, P, C.c_int]),
    "umans_scenario_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "umans_cost_functions": (C.c_int, [C.POINTER(C.c_char_p), C.c_int, C.POINTER(C.c_int)]),
    "umans_scenario_warnings": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_int)]),
    "umans_diff_begin": (C.c_int, [P, C.c_int, C.c_int, P, C.c_float]),
    "umans_diff_forward": (C.c_int, [P, C.POINTER(C.c_double)]),
    "umans_diff_backward": (C.c_int, [P, P, P, P]),
    "umans_diff_end": (C.c_int, [P]),
    "umans_set_force_params": (C.c_int, [P, C.c_int, P]),
    "umans_get_force_params": (C.c_int, [P, C.c_int, P]),
    "umans_record_start": (C.c_int, [P, C.c_char_p, C.c_int, C.c_int]),
    "umans_record_flush": (C.c_int, [P]),
    "umans_record_stop": (C.c_int, [P]),
    "umans_debug_ref_expf": (C.c_int, [P, P, C.c_int, C.POINTER(C.c_size_t)]),
    "umans_debug_ref_sincosf": (C.c_int, [P, P, P, C.c_int, C.POINTER(C.c_size_t)]),
    "umans_debug_expf_check": (C.c_int, [C.c_uint, C.c_uint, P, C.POINTER(C.c_float)]),
    "umans_debug_prod_diff": (C.c_int, [P, P, C.c_int]),
    "umans_orca_velocities_noalloc": (C.c_int, [C.c_int, P, P, P, P, P, P, P, P, P, C.c_int, C.c_float,
                                                C.c_float, C.c_float, C.c_float, P, P]),
    "umans_last_error": (C.c_char_p, [P]),
}

_lib = None


def exported_symbols() -> list[str]:
    return list(_SIGS)


def load(build_if_missing: bool = False):
    """Returns the loaded library; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build
            build.build()
        else:
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA engine first (python -m umans_gb300.build); "
                "there is no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
