"""Binary CSR fixture I/O in the reference's file format.

Format (writer: PythonRef/solve.py:574-676, generator_banded.py:70-172;
reader: matrix_LoadCSR, OpenMP/spike_matrix.c:11-51):

    int32 n, int32 nnz, int32 dtype (0 = float64, 1 = complex128),
    values, int32 colind[nnz], int32 rowptr[n+1]

For dtype 1 the values are *planar*: all nnz real parts, then all nnz
imaginary parts (the writers store ``M.data.real`` then ``M.data.imag``).  The
reference's C loader ignores the flag and reads interleaved pairs
(OpenMP/spike_matrix.c:30-35); this loader honours it.

``save_csr`` writes the dtype flag from the value type (the reference's
``matrix_SaveCSR`` writes its matrix-type field there instead,
OpenMP/spike_matrix.c:71).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np


@dataclass
class CSR:
    n: int
    rowptr: np.ndarray  # int32 [n+1]
    colind: np.ndarray  # int32 [nnz]
    aij: np.ndarray     # float64 or complex128 [nnz]

    @property
    def nnz(self) -> int:
        return int(self.colind.shape[0])

    def to_dense(self) -> np.ndarray:
        A = np.zeros((self.n, self.n), dtype=self.aij.dtype)
        for r in range(self.n):
            s, e = self.rowptr[r], self.rowptr[r + 1]
            A[r, self.colind[s:e]] = self.aij[s:e]
        return A


def load_csr(path: str) -> CSR:
    with open(path, "rb") as f:
        raw = f.read()
    n, nnz, dtype = struct.unpack_from("<iii", raw, 0)
    if n < 0 or nnz < 0 or dtype not in (0, 1):
        raise ValueError(f"{path}: bad header n={n} nnz={nnz} dtype={dtype}")
    off = 12
    if dtype == 1:
        re = np.frombuffer(raw, np.float64, nnz, off)
        off += 8 * nnz
        im = np.frombuffer(raw, np.float64, nnz, off)
        off += 8 * nnz
        aij = (re + 1j * im).astype(np.complex128)
    else:
        aij = np.frombuffer(raw, np.float64, nnz, off).copy()
        off += 8 * nnz
    colind = np.frombuffer(raw, np.int32, nnz, off).copy()
    off += 4 * nnz
    rowptr = np.frombuffer(raw, np.int32, n + 1, off).copy()
    off += 4 * (n + 1)
    if off != len(raw):
        raise ValueError(f"{path}: {len(raw) - off} trailing bytes")
    return CSR(n, rowptr, colind, aij)


def save_csr(path: str, A: CSR) -> None:
    cplx = np.iscomplexobj(A.aij)
    with open(path, "wb") as f:
        f.write(struct.pack("<iii", A.n, A.nnz, 1 if cplx else 0))
        if cplx:
            f.write(np.ascontiguousarray(A.aij.real, np.float64).tobytes())
            f.write(np.ascontiguousarray(A.aij.imag, np.float64).tobytes())
        else:
            f.write(np.ascontiguousarray(A.aij, np.float64).tobytes())
        f.write(np.ascontiguousarray(A.colind, np.int32).tobytes())
        f.write(np.ascontiguousarray(A.rowptr, np.int32).tobytes())
