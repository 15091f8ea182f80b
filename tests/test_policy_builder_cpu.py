"""Policies built in code (Policy / SamplingParameters / add_cost_function)
write the <Policy> elements the loader reads: the benchmark policies rebuilt
this way equal their XML templates attribute for attribute, and a scenario
holding Policy objects loads.  Host only."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from umans_gb300 import Policy, SamplingParameters, cost_functions, scenario_info, scenarios as S

BUILT_IN = ["ORCA", "RVO", "SocialForcesAvoidance", "PowerLaw", "GoalReachingForce", "Karamouzas",
            "Moussaid", "Paris", "VanToll", "TtcaDca", "FOEAvoidance", "PLEdestrians",
            "RandomFunction", "Generic"]


def test_registry_lists_built_ins_then_plugins():
    names = cost_functions()
    assert names[:len(BUILT_IN)] == BUILT_IN
    assert "ExampleRVO" in names[len(BUILT_IN):]


def _same_element(a: str, b: str):
    ea, eb = ET.fromstring(a), ET.fromstring(b)
    assert ea.tag == eb.tag and ea.attrib == eb.attrib
    assert [(c.tag, c.attrib) for c in ea] == [(c.tag, c.attrib) for c in eb]


def test_builder_reproduces_benchmark_policies():
    orca = Policy(0, "global", relaxation_time=0).add_cost_function("ORCA", range=8, timeHorizon=5)
    _same_element(orca.to_xml(), S.ORCA_POLICY.format(pid=0))

    sf = (Policy(1, "gradient", relaxation_time=0.5)
          .add_cost_function("SocialForcesAvoidance", range=5)
          .add_cost_function("GoalReachingForce"))
    _same_element(sf.to_xml(), S.SF_POLICY.format(pid=1, sfparams=""))

    pl = (Policy(2, "sampling", SamplingParameters(type="regular", base="zero", base_direction="unit",
                                                   angle=360, speed_samples=4, angle_samples=36,
                                                   radius="maximum speed"), relaxation_time=0.5)
          .add_cost_function("PowerLaw", range=5).add_cost_function("GoalReachingForce"))
    _same_element(pl.to_xml(), S.POWERLAW_SAMPLING_POLICY.format(pid=2))

    ka = Policy(3, "sampling", SamplingParameters(type="regular", base="zero",
                                                  base_direction="preferred velocity", angle=180,
                                                  speed_samples=10, angle_samples=20,
                                                  include_base_as_sample=True, radius="maximum speed"),
                relaxation_time=0).add_cost_function("Karamouzas", range=10)
    _same_element(ka.to_xml(), S.KARAMOUZAS_POLICY.format(pid=3))


def test_global_fallback_sampling_values():
    p = SamplingParameters.approximate_global_optimization()
    assert p.attributes() == {"SamplingType": "regular", "SamplingBase": "zero",
                              "SamplingBaseDirection": "unit", "SamplingRadius": "maximum speed",
                              "SamplingAngle": "360", "SpeedSamples": "11", "AngleSamples": "36",
                              "IncludeBaseAsSample": "true"}


def test_scenario_with_policy_objects_loads(tmp_path):
    sc = S.model_crossing("RVO")
    sc.policies = [Policy(0, "sampling", SamplingParameters(type="random", random_samples=50),
                          relaxation_time=0.2, contact_force_scale=100)
                   .add_cost_function("ExampleRVO", range=5, w=2)
                   .add_cost_function("RandomFunction", coeff=0.1)]
    sc.policy_id = np.zeros(sc.n, np.int64)
    assert scenario_info(sc.write(str(tmp_path / "p.xml"))) == dict(agents=sc.n, policies=1, edges=0)


def test_builder_errors():
    with pytest.raises(ValueError, match="optimization method"):
        Policy(0, "annealing")
    with pytest.raises(ValueError, match="sampling method only"):
        Policy(0, "gradient", SamplingParameters())
    with pytest.raises(ValueError, match="sampling radius"):
        SamplingParameters(radius="half speed")
    with pytest.raises(ValueError, match="not registered"):
        Policy(0, "gradient").add_cost_function("NoSuchCost")
    p = Policy(0, "gradient")
    for _ in range(4):
        p.add_cost_function("GoalReachingForce")
    with pytest.raises(ValueError, match="more than 4"):
        p.add_cost_function("GoalReachingForce")
    with pytest.raises(ValueError, match="at least one cost function"):
        Policy(1, "global").to_xml()


def test_built_policies_simulate_like_templates(tmp_path):
    """The same crowd under the Karamouzas sampling policy written from its
    template and built in code: identical oracle trajectories."""
    from oracle.port import PortSim
    a = S.model_crossing("RVO")
    a.policies = [S.KARAMOUZAS_POLICY.format(pid=0)]
    b = S.model_crossing("RVO")
    b.policies = [Policy(0, "sampling", SamplingParameters(type="regular", base="zero",
                                                           base_direction="preferred velocity", angle=180,
                                                           speed_samples=10, angle_samples=20,
                                                           include_base_as_sample=True, radius="maximum speed"),
                         relaxation_time=0).add_cost_function("Karamouzas", range=10)]
    sa = PortSim(a.write(str(tmp_path / "a.xml")), threads=2)
    sb = PortSim(b.write(str(tmp_path / "b.xml")), threads=2)
    sa.step(30)
    sb.step(30)
    pa, pb = sa.state()["pos"], sb.state()["pos"]
    assert np.array_equal(pa, pb)
    assert float(np.abs(pa - a.pos).max()) > 0.5   # the crowd moved
