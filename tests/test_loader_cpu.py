"""The scenario loader of the engine library on the host (no device work):
counts, errors, and a large agents block loading in linear time."""
import os
import subprocess
import sys
import textwrap
import time

import pytest

from umans_gb300 import UmansError, scenario_info, scenario_warnings, scenarios as S


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


def test_loader_warnings(tmp_path):
    """Recoverable problems load with the reference's defaults and are
    reported as warnings (crowdSimulator.cpp:344-400)."""
    p = tmp_path / "w.xml"
    p.write_text('<?xml version="1.0"?><Simulation delta_time="0.1"><World type="Spherical"/>'
                 '<Policies><Policy id="3" OptimizationMethod="sampling" SamplingType="jittered">'
                 '<costfunction name="RVO"/><costfunction name="NoSuchCost"/></Policy></Policies>'
                 '<Agents><Agent><pos x="0" y="0"/><Policy id="3"/></Agent></Agents></Simulation>')
    w = scenario_warnings(str(p))
    assert "Policy 3: sampling type invalid, using default (regular)" in w
    assert "Policy 3: unknown cost function NoSuchCost ignored" in w
    assert "agent has no goal element and will not move" in w
    assert "no valid world type; using Infinite" in w
    assert scenario_warnings(S.model_crossing("RVO").write(str(tmp_path / "ok.xml"))) == []
    # a short buffer is filled and terminated, the full size reported
    import ctypes as C
    from umans_gb300 import _lib
    buf, need = C.create_string_buffer(b"\xff" * 8), C.c_int()
    assert _lib.load().umans_scenario_warnings(str(p).encode(), buf, 6, C.byref(need)) == 0
    assert buf.raw[:6] == w[0].encode()[:5] + b"\0" and buf.raw[6:8] == b"\xff\xff"
    assert need.value == len("\n".join(w)) + 2
    with pytest.raises(UmansError):
        scenario_warnings(str(tmp_path / "missing.xml"))


def test_loader_errors(tmp_path):
    p = tmp_path / "bad.xml"
    p.write_text('<?xml version="1.0"?><Simulation delta_time="0.1"><World type="Infinite"/>'
                 '<Agents><Agent><pos x="0" y="0"/><Policy id="0"/></Agent></Agents></Simulation>')
    with pytest.raises(UmansError):
        scenario_info(str(p))
    with pytest.raises(UmansError):
        scenario_info(str(tmp_path / "missing.xml"))


_MUTATE = textwrap.dedent("""
    import ctypes as C, random, sys
    from umans_gb300 import _lib, scenarios as S
    lib = _lib.load()
    rng = random.Random(int(sys.argv[1]))
    base = [S.model_block_field("SocialForces").to_xml().encode(),
            S.model_arrivals("ORCA").to_xml().encode(),
            S.model_toric_obstacle("RVO").to_xml().encode()]
    toks = [b"<", b">", b"/", b'"', b"=", b"<!--", b"-->", b"<?", b"?>", b"&amp;", b"&", b"\\x00",
            b"nan", b"inf", b"-1e39", b"<Agent>", b"</Agent>", b'<Policy id="0">', b"</Policy>",
            b"<Obstacle>", b'<Point x="1" y="1"/>', b'id="-5"', b'width="0"', b'delta_time="0"',
            b"<![CDATA[", b'SpeedSamples="-3"', b"<costfunction/>"]
    a, p, e = C.c_int(), C.c_int(), C.c_int()
    loaded = 0
    for it in range(int(sys.argv[2])):
        d = bytearray(rng.choice(base))
        for _ in range(rng.randint(1, 6)):
            op, pos = rng.random(), rng.randrange(len(d) + 1)
            if op < 0.35: del d[pos:pos + rng.randint(1, 40)]
            elif op < 0.7: d[pos:pos] = rng.choice(toks)
            elif len(d): d[pos % len(d)] = rng.randrange(256)
        if rng.random() < 0.1: d = d[:rng.randrange(len(d) + 1)]
        with open(sys.argv[3], "wb") as fh: fh.write(bytes(d))
        rc = lib.umans_scenario_info(sys.argv[3].encode(), C.byref(a), C.byref(p), C.byref(e))
        assert rc in (0, 2), rc   # UMANS_OK or UMANS_ERR_LOAD
        loaded += rc == 0
    print("loaded", loaded)
""")


@pytest.mark.parametrize("seed", [1, 2])
def test_mutated_files_load_or_fail_cleanly(seed, tmp_path):
    """Seeded byte-level mutations of valid scenario files (deleted spans,
    inserted markup, flipped bytes, truncation): the native loader either
    loads or returns an error status, never crashes.  Runs in a child process
    so that a crash fails this test only."""
    env = dict(os.environ, PYTHONPATH=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    r = subprocess.run([sys.executable, "-c", _MUTATE, str(seed), "400", str(tmp_path / "m.xml")],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("loaded")
