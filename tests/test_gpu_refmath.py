"""The device exponential of the force models equals the host C library's
expf bit for bit on [-87, 0], and the device sine and cosine equal the host
sinf/cosf on [-64, 64] (float-float evaluation + exception tables)."""
import ctypes as C

import numpy as np
import pytest

from oracle.port import libm_expf, libm_sincosf
from umans_gb300 import _lib

pytestmark = pytest.mark.gpu


def device_expf(x):
    lib = _lib.load()
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    cnt = C.c_size_t()
    rc = lib.umans_debug_ref_expf(x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), x.size, C.byref(cnt))
    assert rc == 0, lib.umans_last_error(None)
    return y, cnt.value


def test_ref_expf_bit_exact_dense_range():
    # 20M consecutive floats below -1 (typical -b/sigma arguments), then below -0.001
    for start in (np.float32(-1.0), np.float32(-0.001), np.float32(-20.0)):
        bits = start.view(np.uint32) + np.arange(20_000_000, dtype=np.uint32)
        x = bits.view(np.float32)
        x = x[(x >= -87.0) & (x <= 0.0)]
        y, nexc = device_expf(x)
        ref = libm_expf(x)
        bad = np.nonzero(y.view(np.uint32) != ref.view(np.uint32))[0]
        assert bad.size == 0, f"{bad.size} mismatches, e.g. x={x[bad[:5]]}"
        assert nexc > 0


def test_short_exponential_on_every_float_of_the_domain():
    """The force models try a short FMA exponential first and fall back to
    the float-float one with the exception table only near rounding
    midpoints.  On all 1.1e9 floats of [-87, 0] its answers equal the
    table-backed results and never concern an argument the table lists; on
    the force models' arguments, [-87, -2^-10], it answers almost always
    (below that most results round to 1.0, a power of two it leaves to the
    fallback)."""
    lib = _lib.load()
    first = int(np.float32(-0.0).view(np.uint32))
    count = int(np.float32(-87.0).view(np.uint32)) - first + 1
    out = np.zeros(3, np.uint64)
    band = C.c_float()
    rc = lib.umans_debug_expf_check(first, count, out.ctypes.data_as(C.c_void_p), C.byref(band))
    assert rc == 0, lib.umans_last_error(None)
    answered, differing, listed = (int(v) for v in out)
    print(f"short exponential: answered {answered} of {count} ({answered / count:.5f}), "
          f"differing {differing}, listed {listed}, table band {band.value:.3g} ulp")
    assert differing == 0 and listed == 0
    lo = int(np.float32(-2.0 ** -10).view(np.uint32))
    count2 = int(np.float32(-87.0).view(np.uint32)) - lo + 1
    rc = lib.umans_debug_expf_check(lo, count2, out.ctypes.data_as(C.c_void_p), None)
    assert rc == 0, lib.umans_last_error(None)
    print(f"on [-87, -2^-10]: answered {int(out[0]) / count2:.5f}")
    assert int(out[1]) == 0 and int(out[2]) == 0
    assert int(out[0]) > 0.99 * count2


def test_ref_expf_random_and_edges():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-87, 0, 2_000_000), -np.exp(rng.uniform(-100, 4, 500_000)),
                        [0.0, -0.0, -87.0, -1e-30, -1e-45]]).astype(np.float32)
    x = x[(x >= -87.0) & (x <= 0.0)]
    y, _ = device_expf(x)
    ref = libm_expf(x)
    bad = np.nonzero(y.view(np.uint32) != ref.view(np.uint32))[0]
    assert bad.size == 0, f"{bad.size} mismatches, e.g. x={x[bad[:5]]} got {y[bad[:5]]} want {ref[bad[:5]]}"


def device_prod_diff(a, b, c, d):
    lib = _lib.load()
    q = np.ascontiguousarray(np.stack([a, b, c, d], 1), np.float32)
    y = np.empty(q.shape[0], np.float32)
    rc = lib.umans_debug_prod_diff(q.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), q.shape[0])
    assert rc == 0, lib.umans_last_error(None)
    return y


def host_prod_diff(a, b, c, d):
    f64 = np.float64
    return (f64(a) * f64(b) - f64(c) * f64(d)).astype(np.float32)


def test_prod_diff_matches_double_then_float():
    """(float)((double)a*b - (double)c*d): random operands over many scales,
    squared differences, rotations of unit vectors, heavy cancellation, and
    results placed next to float rounding midpoints."""
    rng = np.random.default_rng(7)
    n = 4_000_000
    cases = []
    f32 = np.float32
    sc = np.exp2(rng.integers(-20, 20, n)).astype(f32)
    cases.append((rng.standard_normal(n).astype(f32) * sc, rng.standard_normal(n).astype(f32),
                  rng.standard_normal(n).astype(f32) * sc, rng.standard_normal(n).astype(f32)))
    x = rng.uniform(0, 20, n).astype(f32)
    y = (x + rng.standard_normal(n).astype(f32) * np.float32(1e-3)).astype(f32)
    cases.append((x, x, y, y))                                   # x^2 - y^2, cancelling
    ang = rng.uniform(-np.pi, np.pi, n)
    cs, sn = np.cos(ang).astype(f32), np.sin(ang).astype(f32)
    v = rng.standard_normal((n, 2)).astype(f32)
    cases.append((cs, v[:, 0], sn, v[:, 1]))                     # rotation, x
    cases.append((sn, v[:, 0], -cs, v[:, 1]))                    # rotation, y
    # a - c*d with c*d about half an ulp of a: results next to midpoints
    a = rng.uniform(1, 2, n).astype(f32)
    ulp = np.spacing(a)
    c = rng.uniform(0.5, 1, n).astype(f32)
    d = (ulp * rng.uniform(0.45, 0.55, n) / c).astype(f32)
    cases.append((a, np.ones(n, f32), c, d))
    for k, (a, b, c, d) in enumerate(cases):
        got = device_prod_diff(a, b, c, d)
        want = host_prod_diff(a, b, c, d)
        bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
        assert bad.size == 0, (k, bad[:5], a[bad[:5]], b[bad[:5]], c[bad[:5]], d[bad[:5]], got[bad[:5]], want[bad[:5]])


def device_sincosf(x):
    lib = _lib.load()
    x = np.ascontiguousarray(x, np.float32)
    s, c = np.empty_like(x), np.empty_like(x)
    cnt = C.c_size_t()
    P = C.c_void_p
    rc = lib.umans_debug_ref_sincosf(x.ctypes.data_as(P), s.ctypes.data_as(P), c.ctypes.data_as(P), x.size,
                                     C.byref(cnt))
    assert rc == 0, lib.umans_last_error(None)
    return s, c, cnt.value


def _check_sincos(x):
    s, c, nexc = device_sincosf(x)
    rs, rc = libm_sincosf(x)
    for name, got, want in (("sin", s, rs), ("cos", c, rc)):
        bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0]
        assert bad.size == 0, f"{name}: {bad.size} mismatches, e.g. x={x[bad[:5]]} got {got[bad[:5]]} want {want[bad[:5]]}"
    return nexc


def test_ref_sincosf_random_sample_angles():
    # the random-sample rotation angles: uniform in [-pi, pi]
    rng = np.random.default_rng(5)
    x = rng.uniform(-np.pi, np.pi, 16_000_000).astype(np.float32)
    assert _check_sincos(x) > 0


def test_ref_sincosf_dense_ranges_and_magnitudes():
    for start in (0.1, 0.7853, 1.0, 1.5707, 3.1415, 40.0, -2.5):
        bits = np.float32(start).view(np.uint32) + np.arange(4_000_000, dtype=np.uint32)
        _check_sincos(bits.view(np.float32))
    rng = np.random.default_rng(6)
    mag = np.exp2(rng.uniform(-20, 6, 8_000_000)).astype(np.float32)
    x = np.where(rng.random(mag.size) < 0.5, -mag, mag).astype(np.float32)
    _check_sincos(x[np.abs(x) <= 64])


def test_ref_sincosf_edges():
    k = np.arange(-40, 41, dtype=np.float64)
    near = (k * np.pi / 2).astype(np.float32)               # floats nearest multiples of pi/2
    near = np.concatenate([near, np.nextafter(near, np.float32(np.inf)), np.nextafter(near, np.float32(-np.inf))])
    x = np.concatenate([near, np.float32([0.0, -0.0, 1e-45, -1e-45, 1e-30, 2.0 ** -12, -(2.0 ** -12), 64.0, -64.0,
                                          np.nextafter(np.float32(2.0 ** -12), np.float32(0))])]).astype(np.float32)
    _check_sincos(x[np.abs(x) <= 64])


FRESH = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from umans_gb300 import Simulation
g = dict(np.load(sys.argv[2]))
open(sys.argv[3], "wb").write(g["xml"].tobytes())
sim = Simulation(sys.argv[3])
done, worst = 0, 0.0
for k, s in enumerate(g["steps"]):
    sim.step(int(s) - done)
    done = int(s)
    worst = max(worst, float(np.abs(sim.positions() - g["pos"][k]).max()))
print(worst)
"""


@pytest.mark.parametrize("name", ["crossing40_RVO", "toric60_Dutra"])
def test_first_simulation_of_a_process_uses_the_tables(name, tmp_path):
    """A process whose first simulation needs the sine tables sets them itself
    (random-sample rotations are detected from the sampling schedule)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    npz = os.path.join(root, "tests", "golden", name + ".npz")
    r = subprocess.run([sys.executable, "-c", FRESH, root, npz, str(tmp_path / "x.xml")], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert float(r.stdout.strip().splitlines()[-1]) == 0.0
