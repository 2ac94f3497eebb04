"""Bandwidth-reducing reordering (spike_rcm_permutation, spike_permute_csr,
spike_permute_vector, spike_dsolve_reordered).

The reference reorders with cuSolverSp's host RCM and csrperm
(OpenMP/spike_cuda.c:898-971) and permutes vectors with permute_vector
(OpenMP/spike_algebra.c:34-53).  Host-side checks run without a GPU: the order
is a permutation, it recovers the band of a scrambled banded matrix as well as
scipy's reverse Cuthill-McKee, B = A(p, p) entry by entry, and the vector
permutation and its inverse.  The GPU test solves a scrambled system.
"""
import numpy as np
import pytest

import hspike_gb300 as hs

sp = pytest.importorskip("scipy.sparse")


def _bandwidth(M):
    M = M.tocoo()
    return int(np.abs(M.row - M.col).max()) if M.nnz else 0


def _scrambled(n, k, seed):
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed)
    A = sp.csr_matrix((a, ci, rp), shape=(n, n))
    q = np.random.default_rng(seed).permutation(n)
    As = A[q][:, q].tocsr()
    As.sort_indices()
    return As, q, xt[:, 0], b[:, 0]


@pytest.mark.parametrize("n,k", [(500, 1), (3000, 5), (4000, 16), (2000, 0)])
def test_rcm_recovers_the_band(n, k):
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    As, q, _, _ = _scrambled(n, k, seed=n + k)
    perm = hs.rcm_permutation(As.indptr, As.indices)
    assert sorted(perm.tolist()) == list(range(n))
    rp, ci, a = hs.permute_csr(As.indptr, As.indices, As.data, perm)
    B = sp.csr_matrix((a, ci, rp), shape=(n, n))
    ref = reverse_cuthill_mckee(As, symmetric_mode=True)
    assert _bandwidth(B) <= max(_bandwidth(As[ref][:, ref]), k)
    assert _bandwidth(B) <= 2 * k + 1
    assert abs(B - As[perm][:, perm]).max() == 0
    assert all(np.all(np.diff(ci[rp[i]:rp[i + 1]]) > 0) for i in range(n))  # rows sorted


def test_rcm_handles_disconnected_components_and_unsymmetric_patterns():
    n = 60
    rows = [i for i in range(n)] + [3, 40, 41]
    cols = [i for i in range(n)] + [57, 2, 10]  # unsymmetric couplings, many isolated nodes
    A = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n))
    A.sort_indices()
    perm = hs.rcm_permutation(A.indptr, A.indices)
    assert sorted(perm.tolist()) == list(range(n))


def test_permute_vector_and_its_inverse():
    rng = np.random.default_rng(1)
    perm = rng.permutation(97).astype(np.int32)
    v = np.asfortranarray(rng.standard_normal((97, 3)))
    w = v.copy(order="F")
    hs.permute_vector(1, perm, w)
    assert np.array_equal(w, v[perm])
    hs.permute_vector(0, perm, w)
    assert np.array_equal(w, v)


def test_invalid_inputs_are_errors():
    with pytest.raises(hs.SpikeError):
        hs.rcm_permutation(np.array([0, 1, 5], np.int32), np.array([0, 1], np.int32))  # rowptr past nnz
    with pytest.raises(hs.SpikeError):
        hs.permute_csr(np.array([0, 1, 2], np.int32), np.array([0, 1], np.int32), np.ones(2),
                       np.array([0, 0], np.int32))  # not a permutation


@pytest.mark.gpu
def test_solve_of_a_scrambled_system():
    from oracle import oracle
    n, k = 20_000, 8
    As, q, xt, b = _scrambled(n, k, seed=7)
    x, perm = hs.solve_reordered(As.indptr, As.indices, As.data, b[q])
    # the scrambled system's solution is x_true(q)
    assert np.linalg.norm(x - xt[q]) / np.linalg.norm(xt) <= 1e-10
    res = oracle.residual(As.indptr.astype(np.int32), As.indices.astype(np.int32), As.data, x[:, None],
                          b[q][:, None]).max()
    assert res <= 1e-12
