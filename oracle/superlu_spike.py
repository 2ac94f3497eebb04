"""SPIKE with SuperLU as the inner solver (test infrastructure only).

A second, independent restatement of the reference's solve
(OpenMP/spike_interfaces.c:43-419) that uses scipy's bundled SuperLU
(``scipy.sparse.linalg.splu``) for every A_i and for the reduced system, the
same family of factorization the reference calls (SuperLU_MT pdgstrf with
partial pivoting, OpenMP/spike_superlu.c:763).  The structure mirrors the
Python prototype's ``spike_implicit_vw`` (PythonRef/spike.py:186-400) with the
C code's tip sizes (top = ku rows, bottom = kl rows) and its schedule
(OpenMP/spike_analysis.c:38-76).  Only tests use it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla


def spike_superlu(rowptr, colind, aij, b, p=4):
    n = len(rowptr) - 1
    A = sp.csr_matrix((aij, colind, rowptr), shape=(n, n))
    b = np.asarray(b)
    b2 = b.reshape(n, -1)
    coo = A.tocoo()
    ku = max(int((coo.col - coo.row).max()), 0)
    kl = max(int((coo.row - coo.col).max()), 0)
    nreg = n // p
    nb = [i * nreg for i in range(p)] + [n]
    s = ku + kl
    R = sp.lil_matrix((p * s, p * s), dtype=b2.dtype if np.iscomplexobj(b2) or np.iscomplexobj(aij) else float)
    R.setdiag(1.0)
    xr = np.zeros((p * s, b2.shape[1]), dtype=R.dtype)
    lus = []
    for q in range(p):
        r0, r1 = nb[q], nb[q + 1]
        m = r1 - r0
        lu = sla.splu(sp.csc_matrix(A[r0:r1, r0:r1]))
        lus.append(lu)
        y = lu.solve(np.ascontiguousarray(b2[r0:r1]).astype(R.dtype))
        xr[q * s:q * s + ku] = y[:ku]
        xr[q * s + ku:(q + 1) * s] = y[m - kl:]
        if q < p - 1:
            V = lu.solve(A[r0:r1, r1:r1 + ku].toarray().astype(R.dtype))
            R[q * s:q * s + ku, (q + 1) * s:(q + 1) * s + ku] = V[:ku]
            R[q * s + ku:(q + 1) * s, (q + 1) * s:(q + 1) * s + ku] = V[m - kl:]
        if q > 0:
            W = lu.solve(A[r0:r1, r0 - kl:r0].toarray().astype(R.dtype))
            R[q * s:q * s + ku, q * s - kl:q * s] = W[:ku]
            R[q * s + ku:(q + 1) * s, q * s - kl:q * s] = W[m - kl:]
    yr = sla.splu(sp.csc_matrix(R)).solve(xr)
    x = np.zeros_like(xr, shape=b2.shape)
    for q in range(p):
        r0, r1 = nb[q], nb[q + 1]
        f = np.array(b2[r0:r1], dtype=R.dtype)
        if q < p - 1:
            f[-ku:] -= A[r1 - ku:r1, r1:r1 + ku] @ yr[(q + 1) * s:(q + 1) * s + ku]
        if q > 0:
            f[:kl] -= A[r0:r0 + kl, r0 - kl:r0] @ yr[q * s - kl:q * s]
        x[r0:r1] = lus[q].solve(f)
    return x.reshape(b.shape) if b.ndim == 2 else x[:, 0]
