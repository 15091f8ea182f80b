"""Host-side checks of the reference-exact arithmetic shared by host and
device code (refmath.hpp): the float-float line intersection never disagrees
with the reference's double pipeline when it decides, and the float-float
sine/cosine differs from the C library only near rounding midpoints; the
tables of the exponential and of the sine/cosine equal what their generators
print."""
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_refmath_host_check(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "refmath_host_check")
    cuda_inc = "/usr/local/cuda/include"
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", cuda_inc, "-o", exe,
                           os.path.join(HERE, "refmath_host_check.cpp"), "-lm"])
    r = subprocess.run([exe, "400000"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    assert "mismatches=0" in lines["isect"]
    assert "unflagged=0" in lines["sincos"]
    assert "mismatches=0" in lines["gauss"]


def _table_rows(header: str, name: str) -> list[str]:
    i = header.index(name)
    body = header[header.index("{", i) + 1:header.index("};", i)]
    return [l.strip() for l in body.strip().splitlines()]


def _generated(script: str) -> list[str]:
    pytest.importorskip("mpmath")
    out = subprocess.run([sys.executable, script], capture_output=True, text=True,
                         check=True).stdout
    return [l.strip() for l in out.strip().splitlines()]


def test_exp2_table_matches_its_generator():
    csrc = os.path.join(HERE, "..", "umans_gb300", "csrc")
    header = open(os.path.join(csrc, "refmath.hpp")).read()
    rows = _generated(os.path.join(csrc, "gen_exp2_table.py"))
    assert len(rows) == 64
    assert _table_rows(header, "FF_EXP2_TAB_D") == rows
    assert _table_rows(header, "FF_EXP2_TAB_H") == rows


def test_sincos_table_matches_its_generator():
    csrc = os.path.join(HERE, "..", "umans_gb300", "csrc")
    header = open(os.path.join(csrc, "refmath.hpp")).read()
    out = _generated(os.path.join(csrc, "gen_sincos_table.py"))
    rows = [l for l in out if l.startswith("{")]
    assert len(rows) == 53
    assert _table_rows(header, "SC_TAB_D") == rows
    assert _table_rows(header, "SC_TAB_H") == rows
    consts = [l for l in out if l.startswith("constexpr float SC_")]
    for c in consts:
        assert c in header, c
