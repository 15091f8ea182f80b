"""Host-side checks of the reference-exact arithmetic shared by host and
device code (refmath.hpp): the float-float line intersection never disagrees
with the reference's double pipeline when it decides, and the float-float
sine/cosine differs from the C library only near rounding midpoints."""
import os
import shutil
import subprocess

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
