"""The C-ABI library builds and exports every function include/*.h declares.

No compute call is made here: these tests run without a GPU."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT
from umans_gb300 import _lib, build


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:bool|int|const char\*|void)\s+\**\s*(\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_reference_functions():
    names = declared_functions()
    for ref_name in ("StartSimulation", "GetSimulationTimeStep", "DoSimulationSteps", "GetAgentPositions",
                     "SetAgentPositions", "AddAgent", "RemoveAgent", "SetAgentGoal", "CleanUp"):
        assert ref_name in names


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} not exported"
    # the Python bindings declare exactly the exported C functions
    assert set(_lib.exported_symbols()) <= set(declared_functions())


def test_agentdata_layout():
    assert ctypes.sizeof(_lib.AgentData) == 28


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load()


_C_CALLER = r"""
#include <stdio.h>
#include "umans_gb300.h"
int main(int argc, char** argv) {
    if (argc < 2) return 9;
    const char* names[64]; int n = 0;
    if (umans_cost_functions(names, 64, &n) != UMANS_OK) return 1;
    int a = 0, p = 0, e = 0;
    if (umans_scenario_info(argv[1], &a, &p, &e) != UMANS_OK) return 2;
    char w[256]; int need = 0;
    if (umans_scenario_warnings(argv[1], w, (int)sizeof w, &need) != UMANS_OK) return 3;
    printf("%d %s %d %d %d %d\n", n, names[0], a, p, e, need);
    return 0;
}
"""


def test_header_is_c99_and_links_from_c(tmp_path):
    """The header compiles as pedantic C99 (what a C or cgo caller sees) and a
    C program linked against the library makes the host-only calls."""
    import shutil
    import subprocess
    from umans_gb300 import scenarios as S
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no gcc")
    lib_dir = os.path.dirname(build.build())
    src, exe = tmp_path / "caller.c", tmp_path / "caller"
    src.write_text(_C_CALLER)
    subprocess.check_call([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                           "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                           "-L", lib_dir, "-lumans_gb300", "-Wl,-rpath," + lib_dir])
    xml = S.model_crossing("RVO").write(str(tmp_path / "c.xml"))
    r = subprocess.run([str(exe), xml], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    n, first, agents, policies, edges, need = r.stdout.split()
    assert first == "ORCA" and int(n) >= 15
    assert (int(agents), int(policies), int(edges), int(need)) == (40, 1, 0, 1)


def test_cost_function_listing_respects_capacity():
    lib = _lib.load()
    buf, n = (ctypes.c_char_p * 4)(), ctypes.c_int()
    buf[3] = b"untouched"
    assert lib.umans_cost_functions(buf, 3, ctypes.byref(n)) == 0
    assert n.value >= 15 and [buf[k] for k in range(4)] == [b"ORCA", b"RVO", b"SocialForcesAvoidance",
                                                              b"untouched"]
    assert lib.umans_cost_functions(None, 1, ctypes.byref(n)) != 0   # names required when cap > 0
