"""Policies built in code, the counterpart of the reference's
``Policy(OptimizationMethod, SamplingParameters)`` and
``Policy::AddCostFunction`` (src/Engine/core/policy.h:100-112, 132-152).

The engine loads policies from the scenario format only, so a ``Policy``
object writes the ``<Policy>`` element that the reference's loader
(``CrowdSimulator::FromConfigFile_loadSinglePolicy``,
src/Engine/core/crowdSimulator.cpp:327-422) reads back into the same policy.
An attribute left at ``None`` is not written, and the loader then applies the
reference's default.  A ``Scenario`` (``umans_gb300.scenarios``) takes
``Policy`` objects in its ``policies`` list beside XML strings.

    p = Policy(0, "sampling", SamplingParameters(type="regular", angle=180,
               speed_samples=10, angle_samples=20, include_base_as_sample=True,
               base_direction="preferred velocity", radius="maximum speed"),
               relaxation_time=0)
    p.add_cost_function("Karamouzas", range=10)
"""
from __future__ import annotations

from dataclasses import dataclass, fields

import numpy as np

MAX_COST_FUNCTIONS = 4          # per policy in this engine (the loader's limit)

# Policy::OptimizationMethodFromString: policy.h:100-111
OPTIMIZATION_METHODS = ("gradient", "sampling", "global")

# SamplingParameters::*FromString: policy.h:39-57
SAMPLING_TYPES = ("regular", "random")
SAMPLING_BASES = ("zero", "current velocity")
SAMPLING_BASE_DIRECTIONS = ("unit", "current velocity", "preferred velocity")
SAMPLING_RADII = ("preferred speed", "maximum speed", "maximum acceleration")


def _num(x) -> str:
    if isinstance(x, (bool, np.bool_)):
        return "true" if x else "false"
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    return "%.9g" % float(np.float32(x))


@dataclass
class SamplingParameters:
    """SamplingParameters (policy.h:36-87).  ``None`` keeps the reference's
    default: regular, base zero, base direction current velocity, radius
    preferred speed, 180 degrees, 4 speeds x 11 angles, 100 random samples,
    base not included (policy.h:59-67)."""
    type: str | None = None
    base: str | None = None
    base_direction: str | None = None
    radius: str | None = None
    angle: float | None = None
    speed_samples: int | None = None
    angle_samples: int | None = None
    random_samples: int | None = None
    include_base_as_sample: bool | None = None

    # XML attribute of each field (crowdSimulator.cpp:344-373)
    _ATTRS = dict(type="SamplingType", base="SamplingBase", base_direction="SamplingBaseDirection",
                  radius="SamplingRadius", angle="SamplingAngle", speed_samples="SpeedSamples",
                  angle_samples="AngleSamples", random_samples="RandomSamples",
                  include_base_as_sample="IncludeBaseAsSample")
    _CHOICES = dict(type=SAMPLING_TYPES, base=SAMPLING_BASES, base_direction=SAMPLING_BASE_DIRECTIONS,
                    radius=SAMPLING_RADII)

    def __post_init__(self):
        for name, allowed in self._CHOICES.items():
            v = getattr(self, name)
            if v is not None and v not in allowed:
                raise ValueError(f"sampling {name} {v!r} is not one of {allowed}")
        for name in ("speed_samples", "angle_samples", "random_samples"):
            v = getattr(self, name)
            if v is not None and int(v) < 0:
                raise ValueError(f"{name} must not be negative")

    @staticmethod
    def approximate_global_optimization() -> "SamplingParameters":
        """The sampling a global-method policy falls back to
        (SamplingParameters::ApproximateGlobalOptimization, policy.h:74-86)."""
        return SamplingParameters(type="regular", base="zero", base_direction="unit",
                                  radius="maximum speed", angle=360, angle_samples=36,
                                  speed_samples=11, include_base_as_sample=True)

    def attributes(self) -> dict:
        return {self._ATTRS[f.name]: _num(v) if not isinstance(v, str) else v
                for f in fields(self) if (v := getattr(self, f.name)) is not None}


class Policy:
    """One navigation policy: an optimisation method, its sampling
    parameters and up to four weighted cost functions."""

    def __init__(self, policy_id: int, method: str, sampling: SamplingParameters | None = None,
                 relaxation_time: float | None = None, contact_force_scale: float | None = None):
        if method not in OPTIMIZATION_METHODS:
            raise ValueError(f"optimization method {method!r} is not one of {OPTIMIZATION_METHODS}")
        if sampling is not None and method != "sampling":
            raise ValueError("sampling parameters are read for the sampling method only")
        self.id = int(policy_id)
        self.method = method
        self.sampling = sampling
        self.relaxation_time = relaxation_time
        self.contact_force_scale = contact_force_scale
        self.cost_functions: list[tuple[str, dict]] = []

    def add_cost_function(self, name: str, coeff: float | None = None, range: float | None = None,
                          **params) -> "Policy":
        """Policy::AddCostFunction (policy.cpp:143-149): a cost function by its
        registered name, its weight, its range and its own parameters (the
        attributes its parseParameters reads).  Returns the policy."""
        from .api import cost_functions
        if name not in cost_functions():
            raise ValueError(f"cost function {name!r} is not registered in this engine")
        if len(self.cost_functions) == MAX_COST_FUNCTIONS:
            raise ValueError(f"more than {MAX_COST_FUNCTIONS} cost functions in a policy")
        attrs = {}
        if coeff is not None:
            attrs["coeff"] = coeff
        if range is not None:
            attrs["range"] = range
        attrs.update(params)
        self.cost_functions.append((name, attrs))
        return self

    def to_xml(self) -> str:
        if not self.cost_functions:
            raise ValueError(f"policy {self.id} needs at least one cost function")
        attrs = {"id": str(self.id), "OptimizationMethod": self.method}
        if self.sampling is not None:
            attrs.update(self.sampling.attributes())
        if self.relaxation_time is not None:
            attrs["RelaxationTime"] = _num(float(self.relaxation_time))
        if self.contact_force_scale is not None:
            attrs["ContactForceScale"] = _num(float(self.contact_force_scale))
        out = "<Policy " + " ".join(f'{k}="{v}"' for k, v in attrs.items()) + ">"
        for name, ca in self.cost_functions:
            out += f'<costfunction name="{name}"' + "".join(
                f' {k}="{v if isinstance(v, str) else _num(v)}"' for k, v in ca.items()) + "/>"
        return out + "</Policy>"
