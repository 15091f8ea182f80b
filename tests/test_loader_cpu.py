"""Scenario generation and the oracle's XML reader (CPU)."""
import numpy as np

from oracle.port import read_scenario
from umans_gb300 import scenarios as S


def test_generators_are_seeded(tmp_path):
    a = S.socialforces_toric(n=500, density=0.625).to_xml()
    b = S.socialforces_toric(n=500, density=0.625).to_xml()
    assert a == b
    assert S.batch_counts().min() >= 8 and S.batch_counts().max() <= 2048


def test_float32_roundtrip(tmp_path):
    sc = S.socialforces_toric(n=200, density=0.625)
    p = sc.write(str(tmp_path / "s.xml"))
    r = read_scenario(p)
    assert np.array_equal(r["pos"], sc.pos)
    assert np.array_equal(r["goal"], sc.goal)
    assert np.array_equal(r["pref_speed"], sc.pref_speed)


def test_lenient_xml_like_tinyxml(tmp_path):
    # a stray root element and a comment with '--' (both occur in the reference's examples)
    (tmp_path / "agents.xml").write_text(
        '<?xml version="1.0"?><Simulation delta_time="0.1"/>\n<Agents>\n<!------ x ------>\n'
        '<Agent><pos x="1" y="2"/><goal x="3" y="4"/><Policy id="7"/></Agent></Agents>')
    (tmp_path / "s.xml").write_text(
        '<Simulation delta_time="0.1"><World type="Infinite"/><Policies>'
        '<Policy id="7" OptimizationMethod="gradient"><costfunction name="NoSuchModel"/>'
        '<costfunction name="GoalReachingForce"/></Policy></Policies>'
        '<Agents file="agents.xml"/></Simulation>')
    r = read_scenario(str(tmp_path / "s.xml"))
    assert len(r["ids"]) == 1 and r["policies"][0].ncost == 1
    assert np.isclose(r["radius"][0], 0.24)
