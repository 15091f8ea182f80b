"""The C++ mirror of the reference's policy and world construction
(include/umans_gb300.hpp: Policy(OptimizationMethod, SamplingParameters),
AddCostFunction, World, over the C ABI): a C++ program builds the benchmark
policies and a scenario with agents and an obstacle; the elements it writes
equal the Python writer's, attribute for attribute, and the loader reads the
file back (host only, no GPU)."""
import os
import shutil
import subprocess
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from umans_gb300 import Policy as PyPolicy, scenario_info, scenarios as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include "umans_gb300.hpp"
#include <cstdio>
#include <iostream>
using namespace umans;
int main(int, char** argv)
{
	// the benchmark policies (SF, ORCA, PowerLaw sampling, Karamouzas)
	Policy sf(1, OptimizationMethod::GRADIENT);
	sf.setRelaxationTime(0.5f);
	sf.AddCostFunction("SocialForcesAvoidance", {}, 5.0f);
	sf.AddCostFunction("GoalReachingForce");
	Policy orca(0, OptimizationMethod::GLOBAL);
	orca.setRelaxationTime(0);
	orca.AddCostFunction("ORCA", { { "timeHorizon", 5.0f } }, 8.0f);
	SamplingParameters ps;
	ps.type = "regular"; ps.base = "zero"; ps.baseDirection = "unit"; ps.angle = 360.0f;
	ps.speedSamples = 4; ps.angleSamples = 36; ps.radius = "maximum speed";
	Policy pl(2, OptimizationMethod::SAMPLING, ps);
	pl.setRelaxationTime(0.5f);
	pl.AddCostFunction("PowerLaw", {}, 5.0f);
	pl.AddCostFunction("GoalReachingForce");
	SamplingParameters ks;
	ks.type = "regular"; ks.base = "zero"; ks.baseDirection = "preferred velocity"; ks.angle = 180.0f;
	ks.speedSamples = 10; ks.angleSamples = 20; ks.includeBaseAsSample = true; ks.radius = "maximum speed";
	Policy ka(3, OptimizationMethod::SAMPLING, ks);
	ka.setRelaxationTime(0);
	ka.AddCostFunction("Karamouzas", {}, 10.0f);
	std::cout << sf.ToXML() << "\n" << orca.ToXML() << "\n" << pl.ToXML() << "\n" << ka.ToXML() << "\n";
	// errors: an unregistered cost function, a fifth cost function
	int errors = 0;
	try { Policy x(9, OptimizationMethod::GRADIENT); x.AddCostFunction("NoSuchCost"); } catch (const std::exception&) { ++errors; }
	try {
		Policy x(9, OptimizationMethod::GRADIENT);
		for (int k = 0; k < 5; ++k) x.AddCostFunction("GoalReachingForce");
	} catch (const std::exception&) { ++errors; }
	std::cout << "errors " << errors << "\n";
	// a toric world with two policies, three agents (one inserted later,
	// removed at its goal) and a square obstacle
	World w(WorldType::Toric, 0.1f, 40, 30);
	w.setEndTime(20);
	w.AddPolicy(sf);
	w.AddPolicy(orca);
	w.AddAgent({ -5, 0 }, { 5, 0.5f }, 1);
	w.AddAgent({ 5, 0 }, { -5, 0 }, 0);
	AgentSpec a;
	a.pos = { 0, 8 }; a.goal = { 0, -8 }; a.radius = 0.25f; a.prefSpeed = 1.1f; a.maxSpeed = 1.6f;
	a.policy = 1; a.startTime = 1.5f; a.removeAtGoal = true;
	w.AddAgent(a);
	w.AddObstacle({ { -1, -1 }, { 1, -1 }, { 1, 1 }, { -1, 1 } });
	w.Write(argv[1]);
	return 0;
}
'''


def _same_element(a, b):
    ea = ET.fromstring(a) if isinstance(a, str) else a
    eb = ET.fromstring(b) if isinstance(b, str) else b
    assert ea.tag == eb.tag and ea.attrib == eb.attrib, (ea.tag, ea.attrib, eb.tag, eb.attrib)
    assert len(ea) == len(eb)
    for x, y in zip(ea, eb):
        _same_element(x, y)


@pytest.fixture(scope="module")
def cpp_run(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("cpp")
    src = d / "world.cpp"
    src.write_text(PROGRAM)
    exe = d / "world"
    lib_dir = os.path.join(ROOT, "umans_gb300")
    subprocess.check_call([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                           str(src), "-o", str(exe), "-L", lib_dir, "-lumans_gb300", "-Wl,-rpath," + lib_dir])
    out_xml = d / "scenario.xml"
    r = subprocess.run([str(exe), str(out_xml)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.splitlines(), str(out_xml)


def test_cpp_policies_equal_the_benchmark_templates(cpp_run):
    lines, _ = cpp_run
    _same_element(lines[0], S.SF_POLICY.format(pid=1, sfparams=""))
    _same_element(lines[1], S.ORCA_POLICY.format(pid=0))
    _same_element(lines[2], S.POWERLAW_SAMPLING_POLICY.format(pid=2))
    _same_element(lines[3], S.KARAMOUZAS_POLICY.format(pid=3))
    assert lines[4] == "errors 2"


def test_cpp_world_equals_the_python_writer_and_loads(cpp_run):
    _, path = cpp_run
    sf = (PyPolicy(1, "gradient", relaxation_time=0.5).add_cost_function("SocialForcesAvoidance", range=5)
          .add_cost_function("GoalReachingForce"))
    orca = PyPolicy(0, "global", relaxation_time=0).add_cost_function("ORCA", range=8, timeHorizon=5)
    sc = S.Scenario(dt=0.1, world="Toric", width=40, height=30, end_time=20, policies=[sf, orca],
                    pos=np.array([[-5, 0], [5, 0], [0, 8]], np.float32),
                    goal=np.array([[5, 0.5], [-5, 0], [0, -8]], np.float32),
                    radius=np.array([0.3, 0.3, 0.25], np.float32), pref_speed=np.array([1.3, 1.3, 1.1], np.float32),
                    max_speed=np.array([1.8, 1.8, 1.6], np.float32), policy_id=np.array([1, 0, 1]),
                    obstacles=[np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], np.float32)],
                    start_time=np.array([0, 0, 1.5], np.float32), remove_at_goal=np.array([False, False, True]))
    _same_element(ET.parse(path).getroot(), ET.fromstring(sc.to_xml().split("\n", 1)[1]))
    info = scenario_info(path)
    assert info == {"agents": 3, "policies": 2, "edges": 4}
