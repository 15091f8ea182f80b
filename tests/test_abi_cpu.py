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
