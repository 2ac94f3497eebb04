"""The CPU oracle pinned against the reference's own known answers.

Golden data (transcribed by tests/golden/make_golden.py from the reference's
Tests/ readmes, fixtures copied byte for byte):
  * penta_10: the full 8x8 reduced system R and its RHS for p = 2, b = 1
    (Tests/spike/penta_10.readme:1-21), pins the reduced-system layout of
    OpenMP/spike_matrix.c:657-740,1414-1495 and the tip placement;
  * solve_small: the solution of tridiagonal.bin with b = 1
    (Tests/solve_small/readme.txt:1-4);
  * bandwidth: ku = 2, kl = 4 (Tests/bandwidth/readme.txt; OpenMP/bandwidth.c:32-41);
  * split: A[0:5,0:5] and A[5:10,5:10] of matrix.bin equal block1/2.bin
    (OpenMP/split.c:43-74).
"""
import json
import os

import numpy as np
import pytest

from hspike_gb300.fixtures import load_csr
from oracle import oracle
from tests.conftest import GOLDEN

G = json.load(open(os.path.join(GOLDEN, "golden.json")))


def fx(name):
    return load_csr(os.path.join(GOLDEN, name))


def test_penta10_reduced_system_matches_reference_readme():
    g = G["penta_10"]
    A = fx(g["file"])
    b = np.full(A.n, g["b"])
    x, R, xr, yr = oracle.spike(A.rowptr, A.colind, A.aij, b, p=g["partitions"], return_reduced=True)
    tol = 0.5 * 10.0 ** (-g["decimals"]) + 1e-12
    np.testing.assert_allclose(R, np.array(g["R"]), rtol=0, atol=tol)
    np.testing.assert_allclose(xr[:, 0], np.array(g["rhs"]), rtol=0, atol=tol)
    xd = np.linalg.solve(A.to_dense(), b)
    # the readme reports a SPIKE error of 3.51E-16 against a direct solve
    assert np.abs(x[:, 0] - xd).max() < 10 * g["spike_error"]
    # the reduced solution equals the tips of the true solution
    ku, kl = oracle.bandwidth(A.rowptr, A.colind)
    nb, rb = oracle.schedule(A.n, 2, ku, kl)
    for q in range(2):
        np.testing.assert_allclose(yr[rb[q]:rb[q] + ku, 0], xd[nb[q]:nb[q] + ku], atol=1e-14)
        np.testing.assert_allclose(yr[rb[q] + ku:rb[q + 1], 0], xd[nb[q + 1] - kl:nb[q + 1]], atol=1e-14)


def test_solve_small_matches_reference_readme():
    g = G["solve_small"]
    A = fx(g["file"])
    b = np.full(A.n, g["b"])
    for p in (1, 2):
        x = oracle.spike(A.rowptr, A.colind, A.aij, b, p=p)[:, 0]
        np.testing.assert_allclose(x, np.array(g["x"]), rtol=0, atol=0.5e-3 + 1e-12)
        rel = oracle.residual(A.rowptr, A.colind, A.aij, x, b)[0]
        assert rel < 1e-15 and rel == pytest.approx(g["relative_residual"], rel=1.0)


def test_bandwidth_matches_reference_readme():
    g = G["bandwidth"]
    A = fx(g["file"])
    assert oracle.bandwidth(A.rowptr, A.colind) == (g["ku"], g["kl"])


def test_split_blocks_match_reference_fixtures():
    g = G["split"]
    A = fx(g["matrix"]).to_dense()
    for name, r0, r1 in g["blocks"]:
        B = fx(name).to_dense()
        np.testing.assert_array_equal(A[r0:r1, r0:r1], B)


def test_schedule_follows_reference_rule():
    # spike_solve_analysis: n[i] = i*floor(n/p), remainder in the last partition
    nb, rb = oracle.schedule(100_003, 4, 2, 3)
    assert list(nb) == [0, 25000, 50000, 75000, 100003]
    assert list(rb) == [0, 5, 10, 15, 20]


@pytest.mark.parametrize("name,p", [("spike__penta_15.bin", 3), ("heptadiagonal__small.bin", 2),
                                    ("heptadiagonal__medium.bin", 4), ("pentadiagonal__small.bin", 2),
                                    ("bandwidth__banded.bin", 2), ("dummy__tridiagonal.bin", 3)])
def test_oracle_spike_equals_dense_solve_on_fixtures(name, p):
    A = fx(name)
    rng = np.random.default_rng(0)
    b = rng.standard_normal((A.n, 3))
    x = oracle.spike(A.rowptr, A.colind, A.aij, b, p=p)
    xd = np.linalg.solve(A.to_dense(), b)
    np.testing.assert_allclose(x, xd, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("name,p", [("spike__penta_15.z", 3), ("complex16__penta_15.z", 2), ("complex16__penta_1k.z", 8)])
def test_oracle_complex_fixtures_planar(name, p):
    A = fx(name)
    assert np.iscomplexobj(A.aij) and np.abs(A.aij.imag).max() > 0
    rng = np.random.default_rng(1)
    b = rng.standard_normal((A.n, 2)) + 1j * rng.standard_normal((A.n, 2))
    x = oracle.spike(A.rowptr, A.colind, A.aij, b, p=p)
    xd = np.linalg.solve(A.to_dense(), b)
    np.testing.assert_allclose(x, xd, rtol=1e-10, atol=1e-12)


def test_oracle_every_column_written():
    # the reference copies column 0 of x_i into every column
    # (OpenMP/spike_matrix.c:1341-1342); the oracle must not
    A = fx("spike__penta_15.bin")
    b = np.stack([np.ones(A.n), np.arange(A.n, dtype=float)], axis=1)
    x = oracle.spike(A.rowptr, A.colind, A.aij, b, p=3)
    assert not np.allclose(x[:, 0], x[:, 1])
    np.testing.assert_allclose(x, np.linalg.solve(A.to_dense(), b), rtol=1e-10, atol=1e-12)


def test_superlu_restatement_agrees():
    """Cross-check with scipy's SuperLU (the reference's inner solver family)."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    sp = pytest.importorskip("scipy.sparse")
    from oracle.superlu_spike import spike_superlu

    import hspike_gb300 as hs

    rp, ci, a, xt, b = hs.gen_banded(3000, 3, 2, 1.3, 11, nrhs=2)
    x1 = oracle.spike(rp, ci, a, b, p=5)
    x2 = spike_superlu(rp, ci, a, b, p=5)
    np.testing.assert_allclose(x1, x2, rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(x1, xt, rtol=1e-10, atol=1e-12)


def test_oracle_on_ragged_random_systems():
    """Random shapes the fixtures do not cover: n not a multiple of p, one-sided
    bands (ku = 0 or kl = 0), ku != kl, p up to n / (2 max(ku, kl)), several
    right-hand sides, real and complex; against a dense solve."""
    import hspike_gb300 as hs

    rng = np.random.default_rng(5)
    for case in range(120):
        n = int(rng.integers(10, 400))
        ku, kl = int(rng.integers(0, 7)), int(rng.integers(0, 7))
        k = max(ku, kl, 1)
        p = int(rng.integers(1, min(max(1, n // (2 * k)), 16) + 1))
        nrhs = int(rng.integers(1, 4))
        rp, ci, a, xt, b = hs.gen_banded(n, ku, kl, 1.2, case, nrhs=nrhs, complex_=case % 3 == 0)
        A = np.zeros((n, n), a.dtype)
        for r in range(n):
            A[r, ci[rp[r]:rp[r + 1]]] = a[rp[r]:rp[r + 1]]
        x = oracle.spike(rp, ci, a, b, p=p).reshape(n, -1)
        xd = np.linalg.solve(A, b.reshape(n, -1))
        assert np.abs(x - xd).max() <= 1e-10 * np.abs(xd).max(), (case, n, ku, kl, p)
