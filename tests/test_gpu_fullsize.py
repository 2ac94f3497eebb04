"""GPU parity at the full sizes of the benchmarked configurations.

The scaled-down parity tests (test_gpu_parity.py) keep every per-partition
shape; these run the configurations themselves, with the same seeds as
bench.py, and hold each result to the solver's bar against the CPU oracle
(oracle/spike_oracle.c, the restated reference path of
OpenMP/spike_interfaces.c:43-419, run with the same partitions):

    relative residual ||b - A x|| / ||b|| <= 1e-12 (FP64, every column)
    ||x - x_oracle|| / ||x_oracle||        <= 1e-9

  * large band: n = 2,000,000, kl = ku = 64, 256 partitions, float64 CSR,
    dominance 1.5, nrhs 1 and 16; mixed precision and plain FP64, device
    arrays, and host arrays through dspike_core_host (twice: the second call
    reuses the plan, leaves the column indices on the host and overlaps the
    copy with the factorization);
  * complex heptadiagonal: n = 4,000,000, kl = ku = 3, complex128, nrhs 4,
    512 partitions, complex64 factors + complex128 refinement.
"""
import numpy as np
import pytest

import hspike_gb300 as hs
from oracle import oracle

pytestmark = pytest.mark.gpu

RES_TOL = 1e-12
ERR_TOL = 1e-9


def relerr(x, ref):
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


@pytest.fixture(scope="module")
def large_band():
    n, k, p = 2_000_000, 64, 256
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, 2, nrhs=1)
    xo = oracle.spike(rp, ci, a, b, p=p)
    return n, k, p, rp, ci, a, xt, b, xo


def _device_solve(torch, ctx, rp, ci, a, b, complex_=False):
    dev = torch.device("cuda:0")
    t_rp, t_ci, t_a = (torch.from_numpy(v).to(dev) for v in (rp, ci, a))
    t_b = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev)
    t_x = torch.zeros_like(t_b)
    n, nrhs = b.shape
    ctx.solve_device(n, len(ci), nrhs, t_ci.data_ptr(), t_rp.data_ptr(), t_a.data_ptr(), t_x.data_ptr(),
                     t_b.data_ptr(), complex_=complex_)
    torch.cuda.synchronize()
    return t_x.cpu().numpy().T


@pytest.mark.parametrize("precision", [hs.SPIKE_PRECISION_MIXED, hs.SPIKE_PRECISION_FP64])
def test_large_band_device_arrays(large_band, precision):
    torch = pytest.importorskip("torch")
    n, k, p, rp, ci, a, xt, b, xo = large_band
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PARTITIONS, p)
    ctx.set_option(hs.SPIKE_OPT_PRECISION, precision)
    x = _device_solve(torch, ctx, rp, ci, a, b)
    info = ctx.info()
    ctx.close()
    assert info.partitions == p and info.block == 64
    # FP32 64-row tiles are eliminated from both ends; FP64 ones (three of
    # them do not fit four CTAs' shared memory) top-down
    assert info.twisted == (precision == hs.SPIKE_PRECISION_MIXED)
    assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
    assert relerr(x, xo) <= ERR_TOL, relerr(x, xo)
    assert relerr(xo, xt) <= 1e-10  # the oracle itself reaches x_true


def test_large_band_host_arrays_through_the_reference_entry_point(large_band):
    n, k, p, rp, ci, a, xt, b, xo = large_band
    hs.set_option(hs.SPIKE_OPT_PARTITIONS, p)
    hs.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_MIXED)
    try:
        for call in range(2):
            x = np.zeros_like(b, order="F")
            assert hs.dspike_core_host(n, len(ci), 1, ci, rp, a, x, b) == hs.SPIKE_SUCCESS, hs.last_error()
            info = hs.get_info()
            assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
            assert relerr(x, xo) <= ERR_TOL, (call, relerr(x, xo))
        assert info.columns_implied == 1  # the reused plan kept the column indices on the host
    finally:
        hs.set_option(hs.SPIKE_OPT_PARTITIONS, 0)


def test_large_band_sixteen_right_hand_sides(large_band):
    torch = pytest.importorskip("torch")
    n, k, p, rp, ci, a, _, _, _ = large_band
    b16 = hs.gen_banded(n, k, k, 1.5, 2, nrhs=16)[4]
    xo = oracle.spike(rp, ci, a, b16, p=p)
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PARTITIONS, p)
    x = _device_solve(torch, ctx, rp, ci, a, b16)
    ctx.close()
    assert oracle.residual(rp, ci, a, x, b16).max() <= RES_TOL
    assert relerr(x, xo) <= ERR_TOL


def test_complex_heptadiagonal_full_size():
    torch = pytest.importorskip("torch")
    n, k, p, nrhs = 4_000_000, 3, 512, 4
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.2, 3, complex_=True, nrhs=nrhs)
    xo = oracle.spike(rp, ci, a, b, p=p)
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PARTITIONS, p)
    x = _device_solve(torch, ctx, rp, ci, a, b, complex_=True)
    info = ctx.info()
    ctx.close()
    assert info.partitions == p
    assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
    assert relerr(x, xo) <= ERR_TOL
    assert relerr(xo, xt) <= 1e-10
