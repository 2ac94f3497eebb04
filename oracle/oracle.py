"""CPU oracle for the SPIKE solve (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (built from ``spike_oracle.c`` by
``oracle/build_oracle.py``) and exposes numpy-friendly wrappers.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module; the product library never does.

The C file restates the reference's ``dspike_core_host``
(OpenMP/spike_interfaces.c:43-419); see its header for the line-by-line map.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib_path() -> str:
    return os.path.join(_HERE, "_build", "liboracle.so")


def _lib():
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            from oracle.build_oracle import build

            build()
        L = C.CDLL(path)
        ip, dp, i64 = C.POINTER(C.c_int), C.c_void_p, C.c_longlong
        L.oracle_bandwidth.argtypes = [C.c_int, ip, ip, ip, ip]
        L.oracle_schedule.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, ip, ip]
        L.oracle_reduced_nnz.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oracle_reduced_nnz.restype = i64
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_set_threads.restype = C.c_int
        for pfx in ("d", "z"):
            f = getattr(L, pfx + "oracle_spike")
            f.argtypes = [C.c_int, C.c_int, C.c_int, ip, ip, dp, dp, dp, C.c_int, ip, ip, dp, dp, dp]
            f.restype = C.c_int
            g = getattr(L, pfx + "oracle_direct")
            g.argtypes = [C.c_int, C.c_int, ip, ip, dp, dp, dp]
            g.restype = C.c_int
            h = getattr(L, pfx + "oracle_residual")
            h.argtypes = [C.c_int, C.c_int, ip, ip, dp, dp, dp, dp]
            h.restype = None
        _LIB = L
    return _LIB


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _vp(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _prep(rowptr, colind, aij, b):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colind = np.ascontiguousarray(colind, dtype=np.int32)
    cplx = np.iscomplexobj(aij) or np.iscomplexobj(b)
    dt = np.complex128 if cplx else np.float64
    aij = np.ascontiguousarray(aij, dtype=dt)
    b = np.asarray(b, dtype=dt)
    if b.ndim == 1:
        b = b[:, None]
    b = np.asfortranarray(b)
    return rowptr, colind, aij, b, ("z" if cplx else "d")


def bandwidth(rowptr, colind):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colind = np.ascontiguousarray(colind, dtype=np.int32)
    ku, kl = C.c_int(), C.c_int()
    _lib().oracle_bandwidth(len(rowptr) - 1, _ip(rowptr), _ip(colind), C.byref(ku), C.byref(kl))
    return ku.value, kl.value


def schedule(n, p, ku, kl):
    nb = np.zeros(p + 1, np.int32)
    rb = np.zeros(p + 1, np.int32)
    if _lib().oracle_schedule(n, p, ku, kl, _ip(nb), _ip(rb)):
        raise ValueError("bad schedule")
    return nb, rb


def set_threads(threads: int) -> int:
    """Threads for the oracle's partition loops (0: the OpenMP default);
    returns the previous limit."""
    return int(_lib().oracle_set_threads(threads))


def spike(rowptr, colind, aij, b, p=4, return_reduced=False):
    """x = A^{-1} b by the restated reference SPIKE path with ``p`` partitions.

    With ``return_reduced`` also returns (R as a dense array, xr, yr), R laid
    out exactly as the reference's reduced system.
    """
    rowptr, colind, aij, b, pfx = _prep(rowptr, colind, aij, b)
    n, nrhs = b.shape
    x = np.zeros_like(b, order="F")
    L = _lib()
    ku, kl = bandwidth(rowptr, colind)
    nR = p * (ku + kl) if p > 1 else 0
    Rp = Rc = Ra = xr = yr = None
    if return_reduced and p > 1:
        nnzR = int(L.oracle_reduced_nnz(p, ku, kl))
        Rp = np.zeros(nR + 1, np.int32)
        Rc = np.zeros(max(nnzR, 1), np.int32)
        Ra = np.zeros(max(nnzR, 1), b.dtype)
        xr = np.zeros((nR, nrhs), b.dtype, order="F")
        yr = np.zeros((nR, nrhs), b.dtype, order="F")
    st = getattr(L, pfx + "oracle_spike")(
        n, len(colind), nrhs, _ip(colind), _ip(rowptr), _vp(aij), _vp(x), _vp(b), p,
        _ip(Rp) if Rp is not None else None, _ip(Rc) if Rc is not None else None,
        _vp(Ra), _vp(xr), _vp(yr))
    if st != 0:
        raise RuntimeError(f"oracle spike failed with status {st}")
    if return_reduced and p > 1:
        R = np.zeros((nR, nR), b.dtype)
        for r in range(nR):
            R[r, Rc[Rp[r]:Rp[r + 1]]] = Ra[Rp[r]:Rp[r + 1]]
        return x, R, xr, yr
    return x


def direct(rowptr, colind, aij, b):
    """Banded LU with partial pivoting on the whole A (the FP64 error oracle)."""
    rowptr, colind, aij, b, pfx = _prep(rowptr, colind, aij, b)
    n, nrhs = b.shape
    x = np.zeros_like(b, order="F")
    st = getattr(_lib(), pfx + "oracle_direct")(n, nrhs, _ip(colind), _ip(rowptr), _vp(aij), _vp(x), _vp(b))
    if st != 0:
        raise RuntimeError(f"oracle direct solve failed with status {st}")
    return x


def residual(rowptr, colind, aij, x, b):
    """Per-column relative residual ||b - A x|| / ||b||, accumulated in double."""
    rowptr, colind, aij, b, pfx = _prep(rowptr, colind, aij, b)
    x = np.asfortranarray(np.asarray(x, dtype=b.dtype).reshape(b.shape, order="F"))
    n, nrhs = b.shape
    out = np.zeros(nrhs, np.float64)
    getattr(_lib(), pfx + "oracle_residual")(n, nrhs, _ip(colind), _ip(rowptr), _vp(aij), _vp(x), _vp(b), _vp(out))
    return out
