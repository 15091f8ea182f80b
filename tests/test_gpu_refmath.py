"""The device exponential of the force models equals the host C library's
expf bit for bit on [-87, 0] (float-float evaluation + exception table)."""
import ctypes as C

import numpy as np
import pytest

from oracle.port import libm_expf
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


def test_ref_expf_random_and_edges():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-87, 0, 2_000_000), -np.exp(rng.uniform(-100, 4, 500_000)),
                        [0.0, -0.0, -87.0, -1e-30, -1e-45]]).astype(np.float32)
    x = x[(x >= -87.0) & (x <= 0.0)]
    y, _ = device_expf(x)
    ref = libm_expf(x)
    bad = np.nonzero(y.view(np.uint32) != ref.view(np.uint32))[0]
    assert bad.size == 0, f"{bad.size} mismatches, e.g. x={x[bad[:5]]} got {y[bad[:5]]} want {ref[bad[:5]]}"
