"""umans_gb300: GB300 engine for the per-step agent update of UMANS
(WorldBase::DoStep).

Python host mirror of the reference's interfaces:

* ``UMANS``       the reference's Python class (src/Library/PyAPI.h:55-246):
                  startSimulation / getSimulationTimeStep / doSimulationSteps /
                  getAgentPositions / setAgentPositions / addAgent /
                  removeAgent / setAgentGoal / cleanUp / getNumberOfAgents.
* ``Simulation``  a handle to one simulation with numpy state access.
* ``Batch``       many independent scenarios stepped together.

Both call the CUDA engine through the C ABI (include/umans_gb300.h).
"""
from ._lib import AgentData  # noqa: F401
from .api import (UMANS, Batch, Simulation, UmansError, cost_functions, read_trajectory,  # noqa: F401
                  scenario_info, scenario_warnings)
from .policy import Policy, SamplingParameters  # noqa: F401

__all__ = ["UMANS", "Simulation", "Batch", "UmansError", "AgentData", "read_trajectory"]
