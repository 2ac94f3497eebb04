"""The FP32 reciprocal of the tile inverses against the correctly rounded one.

The FP32 block LU inverts its pivots with sc_rcp_fast (spike_common.cuh): the
hardware approximation rcp.approx.ftz.f32 refined by one Newton-Raphson step.
Its contract: within 1 ulp of the correctly rounded 1/a (__frcp_rn, and numpy's
float32 division, which is also correctly rounded) for every a whose
reciprocal is a normal float -- the diagonal blocks of a diagonally dominant
matrix never produce other pivots, and the FP64 refinement absorbs the
difference.  Checked on random magnitudes over the whole normal range, both
signs, powers of two and the mantissa extremes.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def _build(tmp_path):
    from hspike_gb300.build import ARCH, nvcc

    so = str(tmp_path / "librcp_check.so")
    subprocess.run([nvcc(), *ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                    "-I", os.path.join(ROOT, "hspike_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "rcp_check.cu"), "-o", so],
                   check=True, capture_output=True, text=True)
    L = C.CDLL(so)
    L.rcp_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.rcp_check.restype = C.c_int
    return L


def _ulps(a, b):
    """distance in representable float32 values (same sign assumed)"""
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


def test_fast_reciprocal_within_one_ulp_of_the_rounded_one(tmp_path):
    L = _build(tmp_path)
    rng = np.random.default_rng(11)
    # reciprocals stay normal: |a| in [2^-125, 2^125]
    mags = np.exp2(rng.uniform(-125.0, 125.0, 1 << 20)).astype(np.float32)
    special = np.array([1.0, 2.0, 0.5, 3.0, 1.5, 0.75, 1.0 - 2 ** -24, 1.0 + 2 ** -23, 2.0 ** 125, 2.0 ** -125,
                        np.nextafter(np.float32(2.0), np.float32(1.0))], np.float32)
    a = np.concatenate([mags, special, np.exp2(np.arange(-125, 126)).astype(np.float32)])
    a = np.concatenate([a, -a]).astype(np.float32)
    fast = np.empty_like(a)
    rn = np.empty_like(a)
    assert L.rcp_check(a.ctypes.data, fast.ctypes.data, rn.ctypes.data, len(a)) == 0
    ref = (np.float32(1.0) / a).astype(np.float32)
    assert np.array_equal(rn, ref)  # __frcp_rn is the correctly rounded reciprocal
    d = _ulps(fast, rn)
    assert d.max() <= 1, (a[d.argmax()], fast[d.argmax()], rn[d.argmax()])
    # powers of two have exact reciprocals: no rounding to miss
    p2 = np.isin(np.abs(a), np.exp2(np.arange(-125, 126)).astype(np.float32))
    assert np.array_equal(fast[p2], rn[p2])
