"""The scenario loader of the engine library on the host (no device work):
counts, errors, and a large agents block loading in linear time."""
import time

import pytest

from umans_gb300 import UmansError, scenario_info, scenarios as S


def test_counts(tmp_path):
    info = scenario_info(S.model_block_field("SocialForces").write(str(tmp_path / "b.xml")))
    assert info == dict(agents=60, policies=1, edges=320)
    info = scenario_info(S.model_arrivals("ORCA").write(str(tmp_path / "a.xml")))
    assert info["agents"] == 40 and info["edges"] == 0


def test_large_agents_block_loads_in_linear_time(tmp_path):
    path = S.karamouzas_corridor(200_000).write(str(tmp_path / "k.xml"))
    t = time.perf_counter()
    info = scenario_info(path)
    t = time.perf_counter() - t
    assert info["agents"] == 200_000
    # a sibling walk restarted from the first child made this quadratic
    # (about 9 s on one x86 core); linear it is well below a second
    assert t < 5.0, t


def test_cost_function_plugin_names(tmp_path):
    """A policy whose only cost function is a plugin loads; an unknown name
    is skipped with a warning, which leaves that policy without costs."""
    def scen(cost):
        return ('<?xml version="1.0"?><Simulation delta_time="0.1"><World type="Infinite"/>'
                '<Policies><Policy id="0" OptimizationMethod="sampling">'
                f'<costfunction name="{cost}" range="5" w="2"/></Policy></Policies>'
                '<Agents><Agent><pos x="0" y="0"/><goal x="5" y="0"/><Policy id="0"/></Agent></Agents>'
                '</Simulation>')
    p = tmp_path / "plugin.xml"
    p.write_text(scen("ExampleRVO"))
    assert scenario_info(str(p)) == dict(agents=1, policies=1, edges=0)
    p.write_text(scen("NoSuchCost"))
    with pytest.raises(UmansError, match="cost function"):
        scenario_info(str(p))


def test_loader_errors(tmp_path):
    p = tmp_path / "bad.xml"
    p.write_text('<?xml version="1.0"?><Simulation delta_time="0.1"><World type="Infinite"/>'
                 '<Agents><Agent><pos x="0" y="0"/><Policy id="0"/></Agent></Agents></Simulation>')
    with pytest.raises(UmansError):
        scenario_info(str(p))
    with pytest.raises(UmansError):
        scenario_info(str(tmp_path / "missing.xml"))
