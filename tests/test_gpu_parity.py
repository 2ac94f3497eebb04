"""GPU parity: the sm_103a SPIKE path against the CPU oracle, through the C ABI.

Bar (the solver's contract): relative residual ||b - A x|| / ||b|| <= 1e-12 in
FP64, and ||x - x_oracle|| / ||x_oracle|| <= 1e-9 against the restated
reference path (oracle/spike_oracle.c) on identical inputs and partitions.
FP32 entry points (sspike/cspike) return float data: their bar is 1e-5.
"""
import json
import os

import numpy as np
import pytest

import hspike_gb300 as hs
from hspike_gb300.fixtures import load_csr
from oracle import oracle
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

RES_TOL = 1e-12
ERR_TOL = 1e-9
MODES = {"mixed": hs.SPIKE_PRECISION_MIXED, "fp64": hs.SPIKE_PRECISION_FP64}


def relerr(x, ref):
    return np.linalg.norm(x - ref) / max(np.linalg.norm(ref), 1e-300)


def check(rp, ci, a, b, p, mode="mixed", x_true=None):
    x = hs.solve(rp, ci, a, b, precision=MODES[mode], partitions=p)
    info = hs.get_info()
    xo = oracle.spike(rp, ci, a, b, p=p)
    xo = xo if np.ndim(b) == 2 else xo[:, 0]
    rr = oracle.residual(rp, ci, a, x, b)
    assert rr.max() <= RES_TOL, (rr, info.refine_sweeps)
    assert info.relres_max <= RES_TOL
    assert relerr(x, xo) <= ERR_TOL
    if x_true is not None:
        xt = x_true if np.ndim(b) == 2 else x_true[:, 0]
        assert relerr(x, xt) <= 1e-10
    return x, info


# ------------------------------------------------------------------ fixtures
@pytest.mark.parametrize("name,p", [("spike__penta_10.bin", 2), ("spike__penta_15.bin", 3),
                                    ("solve_small__tridiagonal.bin", 2), ("bandwidth__banded.bin", 1),
                                    ("heptadiagonal__medium.bin", 2), ("pentadiagonal__small.bin", 1)])
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_reference_fixtures(name, p, mode):
    A = load_csr(os.path.join(GOLDEN, name))
    rng = np.random.default_rng(3)
    b = rng.standard_normal((A.n, 2))
    check(A.rowptr, A.colind, A.aij, b, p, mode)


def test_penta10_golden_solution():
    g = json.load(open(os.path.join(GOLDEN, "golden.json")))["penta_10"]
    A = load_csr(os.path.join(GOLDEN, g["file"]))
    b = np.full(A.n, g["b"])
    for mode in ("mixed", "fp64"):
        x, _ = check(A.rowptr, A.colind, A.aij, b, 2, mode)
        # the reference prints a SPIKE error of 3.51E-16 for its FP64 pivoted
        # solve; the contract here is relres <= 1e-12, so the error against the
        # dense solve is bounded by cond(A) * 1e-12 (cond(A) < 10 for penta_10)
        assert np.abs(x - np.linalg.solve(A.to_dense(), b)).max() < 1e-11


@pytest.mark.parametrize("name,p", [("spike__penta_15.z", 3), ("complex16__penta_1k.z", 8)])
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_reference_complex_fixtures(name, p, mode):
    A = load_csr(os.path.join(GOLDEN, name))
    rng = np.random.default_rng(4)
    b = rng.standard_normal((A.n, 3)) + 1j * rng.standard_normal((A.n, 3))
    check(A.rowptr, A.colind, A.aij, b, p, mode)


# ------------------------------------------------------------------ generated
CASES = [
    # n, ku, kl, dom, p, nrhs
    (1000, 1, 1, 2.0, 4, 1),
    (4099, 2, 2, 2.0, 4, 1),
    (10007, 3, 3, 1.2, 16, 4),
    (6000, 3, 1, 1.5, 7, 2),      # ku != kl
    (20011, 8, 8, 1.5, 32, 1),
    (20000, 16, 16, 1.5, 24, 3),
    (30001, 32, 32, 1.5, 20, 1),
    (40003, 64, 64, 1.5, 16, 1),
    (40000, 64, 64, 1.5, 16, 16),
    (50000, 40, 40, 1.5, 12, 2),  # k not a power of two: padded tile
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"n{c[0]}_k{c[1]}_{c[2]}_p{c[4]}_r{c[5]}")
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_generated_real(case, mode):
    n, ku, kl, dom, p, nrhs = case
    rp, ci, a, xt, b = hs.gen_banded(n, ku, kl, dom, seed=100 + n, nrhs=nrhs)
    check(rp, ci, a, b, p, mode, x_true=xt)


# bands above 64 use 128-row tiles: real data, mixed precision only
CASES_128 = [
    (40000, 100, 100, 1.5, 12, 1),
    (30011, 128, 128, 1.5, 8, 2),
    (25000, 65, 90, 1.5, 9, 1),    # ku != kl
    (20000, 128, 128, 1.5, 6, 33),  # two right-hand-side chunks of 32
    (9000, 72, 72, 1.5, 1, 1),      # one partition
]


@pytest.mark.parametrize("case", CASES_128, ids=lambda c: f"n{c[0]}_k{c[1]}_{c[2]}_p{c[4]}_r{c[5]}")
def test_generated_real_128_row_tiles(case):
    n, ku, kl, dom, p, nrhs = case
    rp, ci, a, xt, b = hs.gen_banded(n, ku, kl, dom, seed=300 + n, nrhs=nrhs)
    x, info = check(rp, ci, a, b, p, "mixed", x_true=xt)
    assert info.block == 128


# partitions eliminated from both ends (tiles 16..64, >= 8 blocks per partition)
CASES_TWIST = [
    (8 * 64 * 4, 64, 64, 1.5, 4, 1),    # exactly 8 blocks per partition
    (9 * 64 * 5 + 37, 64, 64, 1.5, 5, 3),  # odd block count, ragged last block
    (40000, 32, 32, 1.5, 10, 2),
    (8 * 32 * 3, 30, 30, 1.5, 3, 1),    # 32-row tiles (one warp per chain), few chains: exactly 8 blocks per partition
    (9 * 32 * 6 + 19, 32, 25, 1.5, 6, 3),  # the same: odd block count, ragged last block, ku != kl
    (8 * 32 * 620, 30, 30, 1.5, 620, 1),     # 32-row tiles, more than 8 chains per SM: 8 blocks
    (9 * 32 * 620 + 19, 32, 25, 1.5, 620, 3),  # the same: odd block count, ragged last block, ku != kl
    (30000, 16, 9, 1.5, 12, 17),        # ku != kl, two right-hand-side chunks
    (60000, 20, 20, 1.2, 1, 1),         # one partition
    (20000, 1, 1, 2.0, 16, 1),          # 2-row tiles on lanes
    (30001, 3, 2, 1.2, 8, 4),           # 4-row tiles on lanes, ku != kl
    (30001, 3, 2, 1.2, 8, 7),           # the same, lane sweeps over two column chunks (4 + 3)
    (20000, 1, 1, 2.0, 16, 6),          # 2-row tiles, two column chunks (4 + 2)
]


@pytest.mark.parametrize("case", CASES_TWIST, ids=lambda c: f"n{c[0]}_k{c[1]}_{c[2]}_p{c[4]}_r{c[5]}")
def test_two_sided_partitions_match_one_sided(case):
    n, ku, kl, dom, p, nrhs = case
    rp, ci, a, xt, b = hs.gen_banded(n, ku, kl, dom, seed=500 + n, nrhs=nrhs)
    x2, info = check(rp, ci, a, b, p, "mixed", x_true=xt)
    assert info.twisted == 1
    hs.set_option(hs.SPIKE_OPT_TWIST, 0)
    try:
        x1, info1 = check(rp, ci, a, b, p, "mixed", x_true=xt)
        assert info1.twisted == 0
    finally:
        hs.set_option(hs.SPIKE_OPT_TWIST, 1)
    assert relerr(x2, x1) <= ERR_TOL


def test_two_sided_partitions_in_plain_fp64():
    rp, ci, a, xt, b = hs.gen_banded(50000, 24, 24, 1.5, seed=77, nrhs=2)
    x, info = check(rp, ci, a, b, 8, "fp64", x_true=xt)
    assert info.twisted == 1 and info.block == 32
    rp, ci, a, xt, b = hs.gen_banded(50000, 3, 3, 1.5, seed=78, nrhs=3)
    x, info = check(rp, ci, a, b, 12, "fp64", x_true=xt)
    assert info.twisted == 1 and info.block == 4


def test_two_sided_factor_handle_and_complex():
    rp, ci, a, xt, b = hs.gen_banded(40000, 12, 12, 1.5, seed=78, complex_=True, nrhs=2)
    x, info = check(rp, ci, a, b, 8, "mixed", x_true=xt)
    assert info.twisted == 1
    for mode in ("mixed", "fp64"):  # complex heptadiagonal on 4-row tiles, both halves on lanes
        rp, ci, a, xt, b = hs.gen_banded(60000, 3, 3, 1.2, seed=79, complex_=True, nrhs=4)
        x, info = check(rp, ci, a, b, 16, mode, x_true=xt)
        assert info.twisted == 1 and info.block == 4
    rp, ci, a, xt, b = hs.gen_banded(80000, 64, 64, 1.5, seed=79, nrhs=1)
    hs.set_option(hs.SPIKE_OPT_PARTITIONS, 16)
    try:
        f = hs.Factor(rp, ci, a)
        try:
            for _ in range(2):
                x = f.solve(b)
                assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
                assert relerr(x, xt) <= 1e-10
        finally:
            f.release()
    finally:
        hs.set_option(hs.SPIKE_OPT_PARTITIONS, 0)


def test_128_row_tiles_auto_partitions_and_factor_reuse():
    rp, ci, a, xt, b = hs.gen_banded(200_000, 96, 96, 1.5, seed=41, nrhs=2)
    x = hs.solve(rp, ci, a, b)
    assert hs.get_info().block == 128 and hs.get_info().partitions > 1
    assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
    assert relerr(x, xt) <= 1e-10
    f = hs.Factor(rp, ci, a)
    try:
        for _ in range(2):
            x2 = f.solve(b)
            assert oracle.residual(rp, ci, a, x2, b).max() <= RES_TOL
    finally:
        f.release()


@pytest.mark.parametrize("case", [(5000, 3, 3, 1.2, 8, 4), (8191, 1, 1, 2.0, 5, 1), (12000, 8, 8, 1.5, 6, 2),
                                  (20000, 32, 32, 1.5, 8, 1)],
                         ids=lambda c: f"n{c[0]}_k{c[1]}_p{c[4]}_r{c[5]}")
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_generated_complex(case, mode):
    n, ku, kl, dom, p, nrhs = case
    rp, ci, a, xt, b = hs.gen_banded(n, ku, kl, dom, seed=7 + n, complex_=True, nrhs=nrhs)
    check(rp, ci, a, b, p, mode, x_true=xt)


def test_single_partition_and_auto_partitions():
    rp, ci, a, xt, b = hs.gen_banded(3000, 4, 4, 1.5, seed=5)
    check(rp, ci, a, b, 1, "mixed", x_true=xt)
    x = hs.solve(rp, ci, a, b, partitions=0)
    assert hs.get_info().partitions >= 1
    assert relerr(x, xt) <= 1e-10


def test_pentadiagonal_100k_on_four_partitions():
    """Plain FP64 SPIKE, 4 partitions, pentadiagonal n = 100,000, 1 RHS, dominance 2.0."""
    rp, ci, a, xt, b = hs.gen_banded(100_000, 2, 2, 2.0, seed=1)
    check(rp, ci, a, b, 4, "fp64", x_true=xt)
    check(rp, ci, a, b, 4, "mixed", x_true=xt)


# ------------------------------------------------------------------ entry points
def test_all_five_entry_points():
    n = 5000
    rp, ci, a, xt, b = hs.gen_banded(n, 3, 3, 1.5, seed=9, nrhs=2)
    hs.set_option(hs.SPIKE_OPT_PARTITIONS, 8)
    hs.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_MIXED)
    x = np.zeros_like(b, order="F")
    assert hs.dspike_core_host(n, len(ci), 2, ci, rp, a, x, b) == hs.SPIKE_SUCCESS
    assert relerr(x, xt) < 1e-10
    x2 = np.zeros_like(b, order="F")
    assert hs.dspike_core_host_blocking(n, len(ci), 2, ci, rp, a, x2, b) == hs.SPIKE_SUCCESS
    np.testing.assert_array_equal(x, x2)
    # single precision in, single precision out
    af, bf = a.astype(np.float32), np.asfortranarray(b.astype(np.float32))
    xf = np.zeros_like(bf, order="F")
    assert hs.sspike_core_host(n, len(ci), 2, ci, rp, af, xf, bf) == hs.SPIKE_SUCCESS
    xo = oracle.spike(rp, ci, af.astype(np.float64), bf.astype(np.float64), p=8)
    assert relerr(xf.astype(np.float64), xo) < 1e-6
    # complex
    rp, ci, a, xt, b = hs.gen_banded(n, 2, 2, 1.5, seed=10, complex_=True, nrhs=2)
    xz = np.zeros_like(b, order="F")
    assert hs.zspike_core_host(n, len(ci), 2, ci, rp, a, xz, b) == hs.SPIKE_SUCCESS
    assert relerr(xz, xt) < 1e-10
    ac, bc = a.astype(np.complex64), np.asfortranarray(b.astype(np.complex64))
    xc = np.zeros_like(bc, order="F")
    assert hs.cspike_core_host(n, len(ci), 2, ci, rp, ac, xc, bc) == hs.SPIKE_SUCCESS
    xo = oracle.spike(rp, ci, ac.astype(np.complex128), bc.astype(np.complex128), p=8)
    assert relerr(xc.astype(np.complex128), xo) < 1e-6
    hs.set_option(hs.SPIKE_OPT_PARTITIONS, 0)


def test_b_not_modified_and_x_overwritten():
    rp, ci, a, xt, b = hs.gen_banded(2000, 2, 2, 2.0, seed=12, nrhs=3)
    b0 = b.copy()
    x = np.full_like(b, np.nan, order="F")
    assert hs.dspike_core_host(2000, len(ci), 3, ci, rp, a, x, b) == hs.SPIKE_SUCCESS
    np.testing.assert_array_equal(b, b0)
    assert np.isfinite(x).all() and relerr(x, xt) < 1e-10


# ------------------------------------------------------------------ factor handles
def test_factor_once_solve_many():
    rp, ci, a, xt, b = hs.gen_banded(30000, 16, 16, 1.5, seed=13)
    f = hs.Factor(rp, ci, a)
    rng = np.random.default_rng(0)
    for nrhs in (1, 3, 70):
        bb = rng.standard_normal((30000, nrhs))
        x = f.solve(bb)
        xo = oracle.direct(rp, ci, a, bb)
        assert relerr(x, xo) <= ERR_TOL
        assert oracle.residual(rp, ci, a, x, bb).max() <= RES_TOL
    f.release()


def test_device_pointer_api_with_torch_stream():
    torch = pytest.importorskip("torch")
    rp, ci, a, xt, b = hs.gen_banded(50000, 8, 8, 1.5, seed=14, nrhs=2)
    dev = torch.device("cuda:0")
    t_rp, t_ci = torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev)
    t_a = torch.from_numpy(a).to(dev)
    t_b = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev)  # column-major n x nrhs
    t_x = torch.zeros_like(t_b)
    ctx = hs.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    ctx.set_option(hs.SPIKE_OPT_PARTITIONS, 32)
    ctx.solve_device(50000, len(ci), 2, t_ci.data_ptr(), t_rp.data_ptr(), t_a.data_ptr(), t_x.data_ptr(),
                     t_b.data_ptr())
    torch.cuda.synchronize()
    x = t_x.cpu().numpy().T
    assert relerr(x, xt) < 1e-10
    assert ctx.info().kernel_launches > 0
    ctx.close()


# ------------------------------------------------------------------ errors
def test_zero_pivot_is_reported_not_trapped():
    rp, ci, a, xt, b = hs.gen_banded(4000, 2, 2, 2.0, seed=15)
    a = a.copy()
    # zero out row 100 entirely: A is singular, block elimination hits a zero pivot
    a[rp[100]:rp[101]] = 0.0
    x = np.zeros_like(b, order="F")
    rc = hs.dspike_core_host(4000, len(ci), 1, ci, rp, a, x, b)
    assert rc == hs.SPIKE_ERROR
    assert hs.ERR_NAMES[hs.last_error()[0]] in ("pivot", "convergence")
    # the context stays usable
    rp, ci, a, xt, b = hs.gen_banded(4000, 2, 2, 2.0, seed=16)
    x = np.zeros_like(b, order="F")
    assert hs.dspike_core_host(4000, len(ci), 1, ci, rp, a, x, b) == hs.SPIKE_SUCCESS


def test_invalid_csr_is_rejected():
    rp, ci, a, xt, b = hs.gen_banded(1000, 2, 2, 2.0, seed=17)
    x = np.zeros_like(b, order="F")
    bad = ci.copy()
    bad[10], bad[11] = bad[11], bad[10]  # unsorted row
    assert hs.dspike_core_host(1000, len(ci), 1, bad, rp, a, x, b) == hs.SPIKE_ERROR
    assert hs.ERR_NAMES[hs.last_error()[0]] == "csr"
    bad = ci.copy()
    bad[5] = 5000  # column out of range
    assert hs.dspike_core_host(1000, len(ci), 1, bad, rp, a, x, b) == hs.SPIKE_ERROR
    assert hs.ERR_NAMES[hs.last_error()[0]] == "csr"
    badp = rp.copy()
    badp[500] = len(ci) + 100  # row pointer past nnz
    assert hs.dspike_core_host(1000, len(ci), 1, ci, badp, a, x, b) == hs.SPIKE_ERROR
    assert hs.ERR_NAMES[hs.last_error()[0]] == "csr"


def test_reused_plan_validates_each_call():
    # a call with the shape (n, nnz) of the previous one skips the separate
    # analysis pass: the band-tile pass validates the CSR and measures the
    # bandwidth, falling back to a new plan when the tile class changed
    ctx = hs.Context()
    try:
        n = 30000
        rp, ci, a, xt, b = hs.gen_banded(n, 10, 10, 1.5, seed=23)
        x1 = hs.solve(rp, ci, a, b, ctx=ctx)
        x2 = hs.solve(rp, ci, a, b, ctx=ctx)
        assert np.array_equal(x1, x2)
        assert (ctx.info().ku, ctx.info().kl, ctx.info().block) == (10, 10, 16)
        # same n and nnz, bandwidth 14: same tile class, the plan is kept
        ci14 = ci.copy()
        ci14[rp[1] - 1] = 14  # row 0's last column 10 -> 14 (still sorted)
        x = hs.solve(rp, ci14, a, b, ctx=ctx)
        assert (ctx.info().ku, ctx.info().kl, ctx.info().block) == (14, 10, 16)
        assert oracle.residual(rp, ci14, a, x, b).max() <= RES_TOL
        # bandwidth 60: another tile class -> a new plan, same answer quality
        ci60 = ci.copy()
        ci60[rp[1] - 1] = 60
        x = hs.solve(rp, ci60, a, b, ctx=ctx)
        assert (ctx.info().ku, ctx.info().block) == (60, 64)
        assert oracle.residual(rp, ci60, a, x, b).max() <= RES_TOL
        hs.solve(rp, ci60, a, b, ctx=ctx)  # reuse that plan
        # invalid CSR with the reused shape: rejected, not misread
        for bad_ci, bad_rp in ((ci60.copy(), rp), (ci60.copy(), rp.copy())):
            if bad_rp is rp:
                bad_ci[100], bad_ci[101] = bad_ci[101], bad_ci[100]  # unsorted row
            else:
                bad_ci[7] = n + 5  # column out of range
            with pytest.raises(hs.SpikeError) as e:
                hs.solve(bad_rp, bad_ci, a, b, ctx=ctx)
            assert e.value.name == "csr"
        bad_rp = rp.copy()
        bad_rp[500] = len(ci) + 100  # row pointer past nnz
        with pytest.raises(hs.SpikeError) as e:
            hs.solve(bad_rp, ci60, a, b, ctx=ctx)
        assert e.value.name == "csr"
        x = hs.solve(rp, ci, a, b, ctx=ctx)  # and back to the first matrix
        assert relerr(x, x1) <= 1e-12
    finally:
        ctx.close()


def test_reused_plan_validates_each_call_small_tiles():
    # the same for 4-row tiles, whose band pass runs one thread per row
    # (k_band_rows): measured bandwidth, rejected CSR, and back
    ctx = hs.Context()
    try:
        n = 40000
        rp, ci, a, xt, b = hs.gen_banded(n, 3, 3, 1.5, seed=29)
        x1 = hs.solve(rp, ci, a, b, ctx=ctx)
        x2 = hs.solve(rp, ci, a, b, ctx=ctx)
        assert np.array_equal(x1, x2)
        assert (ctx.info().ku, ctx.info().kl, ctx.info().block) == (3, 3, 4)
        assert relerr(x1, oracle.spike(rp, ci, a, b, p=ctx.info().partitions)) <= ERR_TOL
        ci4 = ci.copy()
        ci4[rp[1] - 1] = 4  # row 0's last column 3 -> 4 (still sorted): ku 4, same tile class
        x = hs.solve(rp, ci4, a, b, ctx=ctx)
        assert (ctx.info().ku, ctx.info().kl, ctx.info().block) == (4, 3, 4)
        assert oracle.residual(rp, ci4, a, x, b).max() <= RES_TOL
        for bad_ci, bad_rp in ((ci.copy(), rp), (ci.copy(), rp.copy())):
            if bad_rp is rp:
                bad_ci[100], bad_ci[101] = bad_ci[101], bad_ci[100]  # unsorted row
            else:
                bad_ci[7] = n + 5  # column out of range
            with pytest.raises(hs.SpikeError) as e:
                hs.solve(bad_rp, bad_ci, a, b, ctx=ctx)
            assert e.value.name == "csr"
        bad_rp = rp.copy()
        bad_rp[500] = len(ci) + 100  # row pointer past nnz
        with pytest.raises(hs.SpikeError) as e:
            hs.solve(bad_rp, ci, a, b, ctx=ctx)
        assert e.value.name == "csr"
        x = hs.solve(rp, ci, a, b, ctx=ctx)
        assert relerr(x, x1) <= 1e-12
    finally:
        ctx.close()


def test_host_arrays_copy_overlaps_factorization():
    # a reference-API call with host arrays and the previous call's shape sends
    # the matrix in partition ranges while each range's factorization runs
    ctx = hs.Context()
    try:
        n = 220000
        rp, ci, a, xt, b = hs.gen_banded(n, 32, 32, 1.5, seed=31, nrhs=2)
        assert len(ci) >= 8 << 20
        x1 = hs.solve(rp, ci, a, b, ctx=ctx)      # plans
        x2 = hs.solve(rp, ci, a, b, ctx=ctx)      # copies overlap the factorization
        assert ctx.info().twisted == 1
        assert relerr(x2, x1) <= 1e-13
        assert oracle.residual(rp, ci, a, x2, b).max() <= RES_TOL
        assert relerr(x2, xt) <= 1e-10
        # a new band class with the same shape: the call re-plans after the copy
        ci60 = ci.copy()
        ci60[rp[1] - 1] = 60
        x = hs.solve(rp, ci60, a, b, ctx=ctx)
        assert ctx.info().block == 64
        assert oracle.residual(rp, ci60, a, x, b).max() <= RES_TOL
        hs.solve(rp, ci60, a, b, ctx=ctx)
        # invalid CSR with the reused shape
        bad = ci60.copy()
        bad[1000], bad[1001] = bad[1001], bad[1000]
        with pytest.raises(hs.SpikeError) as e:
            hs.solve(rp, bad, a, b, ctx=ctx)
        assert e.value.name == "csr"
        badp = rp.copy()
        badp[n // 2] = len(ci) + 7
        with pytest.raises(hs.SpikeError) as e:
            hs.solve(badp, ci60, a, b, ctx=ctx)
        assert e.value.name == "csr"
        x = hs.solve(rp, ci60, a, b, ctx=ctx)
        assert oracle.residual(rp, ci60, a, x, b).max() <= RES_TOL
        # complex data through the same path (zspike_core_host semantics)
        rp, ci, a, xt, b = hs.gen_banded(220000, 20, 20, 1.5, seed=32, complex_=True, nrhs=1)
        assert len(ci) >= 8 << 20
        for _ in range(2):
            x = hs.solve(rp, ci, a, b, ctx=ctx)
            assert ctx.info().twisted == 1
            assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
            assert relerr(x, xt) <= 1e-10
    finally:
        ctx.close()


@pytest.mark.parametrize("n,k,nrhs,complex_,mode,twist",
                         [(300_000, 8, 1, False, "mixed", 1), (300_000, 24, 40, False, "mixed", 1),
                          (300_000, 24, 3, False, "mixed", 0), (280_000, 3, 2, True, "mixed", 1),
                          (280_000, 16, 2, False, "fp64", 1), (262_144, 100, 1, False, "mixed", 1)],
                         ids=lambda v: str(v))
def test_reduced_factorization_beside_first_sweep(n, k, nrhs, complex_, mode, twist):
    # from 2^18 rows the reduced factorization runs on a second stream beside
    # the first right-hand-side sweep; with phase timing the two run one after
    # the other: the same kernels on the same data, so x is bit-identical
    # (from 8M entries the reused plan's call also sends the matrix in ranges,
    # whose factorization sums in another order: there 1e-13)
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed=900 + k, complex_=complex_, nrhs=nrhs)
    ctx = hs.Context()
    try:
        ctx.set_option(hs.SPIKE_OPT_TWIST, twist)
        xs = []
        for timing in (0, 0, 1):  # plan; reused plan; serialised phases
            ctx.set_option(hs.SPIKE_OPT_PHASE_TIMING, timing)
            xs.append(hs.solve(rp, ci, a, b, precision=MODES[mode], ctx=ctx))
            assert ctx.info().relres_max <= RES_TOL
        if not twist or k > 64:
            assert ctx.info().twisted == 0
        assert np.array_equal(xs[0], xs[2])
        if len(ci) < 8 << 20:
            assert np.array_equal(xs[1], xs[2])
        else:
            assert relerr(xs[1], xs[2]) <= 1e-13
        assert xs[0].shape == xt.shape == (n, nrhs)
        assert oracle.residual(rp, ci, a, xs[0], b).max() <= RES_TOL
        assert relerr(xs[0], xt) <= 1e-10
    finally:
        ctx.close()


def test_host_arrays_full_band_columns_stay_on_host():
    # a reused plan's call with host arrays checks on host threads that the CSR
    # is the full band while the values travel; the column indices then never
    # cross the host link, and the results equal those of the copied columns
    ctx = hs.Context()
    try:
        n, k = 220000, 30
        rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed=33, nrhs=2)
        assert len(ci) >= 8 << 20
        hs.solve(rp, ci, a, b, ctx=ctx)                       # plans
        x_imp = hs.solve(rp, ci, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 1 and ctx.info().twisted == 1
        assert (ctx.info().ku, ctx.info().kl) == (k, k)
        ctx.set_option(hs.SPIKE_OPT_HOST_THREADS, 0)
        x_cols = hs.solve(rp, ci, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 0
        ctx.set_option(hs.SPIKE_OPT_HOST_THREADS, 8)
        assert np.array_equal(x_imp, x_cols)
        assert oracle.residual(rp, ci, a, x_imp, b).max() <= RES_TOL
        assert relerr(x_imp, xt) <= 1e-10
        # one row past the middle reaches one column further left: the ranges
        # before it keep implied columns, the rest are sent and validated
        r = int(n * 0.7)
        ci2 = ci.copy()
        ci2[rp[r]] = r - k - 1
        x2 = hs.solve(rp, ci2, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 0
        assert (ctx.info().ku, ctx.info().kl) == (k, k + 1)
        assert oracle.residual(rp, ci2, a, x2, b).max() <= RES_TOL
        # the band of the new plan (kl = k + 1) is not the full band either
        x2b = hs.solve(rp, ci2, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 0 and np.array_equal(x2, x2b)
        # back to the full band (kl = k, within the plan's tile class)
        x3 = hs.solve(rp, ci, a, b, ctx=ctx)
        assert oracle.residual(rp, ci, a, x3, b).max() <= RES_TOL
        x3 = hs.solve(rp, ci, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 1 and np.array_equal(x3, x_imp)
        # an unsorted row in the middle is still caught (on the device, after the check fails)
        bad = ci.copy()
        q = rp[int(n * 0.4)] + 5
        bad[q], bad[q + 1] = bad[q + 1], bad[q]
        with pytest.raises(hs.SpikeError) as e:
            hs.solve(rp, bad, a, b, ctx=ctx)
        assert e.value.name == "csr"
        # complex data, then a band break in it (a row reaching one column further)
        rp, ci, a, xt, b = hs.gen_banded(200000, 24, 24, 1.5, seed=34, complex_=True, nrhs=1)
        assert len(ci) >= 8 << 20
        for _ in range(2):
            x = hs.solve(rp, ci, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 1
        assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
        assert relerr(x, xt) <= 1e-10
        r = 150000
        ci3 = ci.copy()
        ci3[rp[r + 1] - 1] = r + 25  # last column r + 24 -> r + 25: still sorted, not the full band
        x = hs.solve(rp, ci3, a, b, ctx=ctx)
        assert ctx.info().columns_implied == 0 and ctx.info().ku == 25
        assert oracle.residual(rp, ci3, a, x, b).max() <= RES_TOL
        # plain FP64 through the same path
        rp, ci, a, xt, b = hs.gen_banded(200000, 24, 24, 1.5, seed=35, nrhs=2)
        for _ in range(2):
            x = hs.solve(rp, ci, a, b, precision=hs.SPIKE_PRECISION_FP64, ctx=ctx)
        assert ctx.info().columns_implied == 1
        assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
        assert relerr(x, xt) <= 1e-12
    finally:
        ctx.close()


def test_bandwidth_above_tile_is_rejected():
    rp, ci, a, xt, b = hs.gen_banded(2000, 130, 130, 1.5, seed=18)
    x = np.zeros_like(b, order="F")
    assert hs.dspike_core_host(2000, len(ci), 1, ci, rp, a, x, b) == hs.SPIKE_ERROR
    assert hs.ERR_NAMES[hs.last_error()[0]] == "bandwidth"
    assert not x.any()


def test_128_row_tiles_only_in_real_mixed_precision():
    rp, ci, a, xt, b = hs.gen_banded(3000, 70, 70, 1.5, seed=19)
    with pytest.raises(hs.SpikeError) as e:
        hs.solve(rp, ci, a, b, precision=hs.SPIKE_PRECISION_FP64)
    assert e.value.name == "bandwidth"
    rp, ci, a, xt, b = hs.gen_banded(3000, 70, 70, 1.5, seed=19, complex_=True)
    x = np.zeros_like(b, order="F")
    assert hs.zspike_core_host(3000, len(ci), 1, ci, rp, a, x, b) == hs.SPIKE_ERROR
    assert hs.ERR_NAMES[hs.last_error()[0]] == "bandwidth"


@pytest.mark.parametrize("n,k,p,nrhs,complex_",
                         [(60_000, 2, 16, 2, False), (80_000, 8, 40, 1, False), (120_000, 32, 24, 3, False),
                          (200_000, 64, 48, 1, False), (90_000, 3, 30, 2, True), (60_000, 100, 12, 1, False)],
                         ids=lambda v: str(v))
def test_reduced_system_in_fp64(n, k, p, nrhs, complex_):
    # SPIKE_OPT_REDUCED_FP64: the reduced system's cyclic reduction in FP64
    # (the reference solves R in FP64 with PARDISO, OpenMP/spike_algebra.c:
    # 263-420) beside FP32 partition factors; 128-row tiles keep their FP32
    # reduced system (the option does not apply there)
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed=700 + k, complex_=complex_, nrhs=nrhs)
    xo = oracle.spike(rp, ci, a, b, p=p)
    ctx = hs.Context()
    try:
        ctx.set_option(hs.SPIKE_OPT_REDUCED_FP64, 1)
        assert ctx.get_option(hs.SPIKE_OPT_REDUCED_FP64) == 1
        for call in range(2):  # new plan, then the reused plan
            x = hs.solve(rp, ci, a, b, precision=hs.SPIKE_PRECISION_MIXED, partitions=p, ctx=ctx)
            info = ctx.info()
            assert info.reduced_fp64 == (1 if k <= 64 else 0)
            assert info.relres_max <= RES_TOL
            assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
            assert relerr(x, xo) <= ERR_TOL
        ctx.set_option(hs.SPIKE_OPT_REDUCED_FP64, 0)
        x32 = hs.solve(rp, ci, a, b, precision=hs.SPIKE_PRECISION_MIXED, partitions=p, ctx=ctx)
        assert ctx.info().reduced_fp64 == 0
        assert relerr(x32, xo) <= ERR_TOL
    finally:
        ctx.close()
