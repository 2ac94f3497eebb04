"""hspike_gb300 -- GB300-native SPIKE banded solver.

The product is the C-ABI library ``_build/libspike_gb300.so`` (C host layer +
sm_103a kernels).  This module is a thin ctypes mirror of its API for Python
callers, tests and the benchmark:

* ``dspike_core_host`` / ``zspike_core_host`` / ``sspike_core_host`` /
  ``cspike_core_host`` / ``dspike_core_host_blocking`` -- the reference's
  entry points (OpenMP/spike_interfaces.h:28-72), same argument order and
  meaning, numpy arrays in place of pointers, ``Error_t`` returned;
* ``Context`` / ``Factor`` / ``Batch`` / ``Server`` -- the extensions of
  ``include/spike_gb300.h``;
* ``solve`` -- convenience wrapper returning x.

There is no Python or CPU compute path: if the library is missing, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import gen_path, lib_path

SPIKE_SUCCESS = 0
SPIKE_ERROR = 1

SPIKE_OPT_PRECISION = 0
SPIKE_OPT_PARTITIONS = 1
SPIKE_OPT_MAX_REFINE = 2
SPIKE_OPT_TOLERANCE = 3
SPIKE_OPT_REDUCED_REFINE = 4
SPIKE_OPT_PHASE_TIMING = 5
PHASES = ["analysis", "factor_fwd", "factor_bwd", "reduced_factor", "rhs_sweeps", "reduced_solve", "retrieval",
          "residual", "band_tiles"]
SPIKE_PRECISION_MIXED = 0
SPIKE_PRECISION_FP64 = 1

ERR_NAMES = {0: "none", 1: "argument", 2: "csr", 3: "bandwidth", 4: "cuda", 5: "memory", 6: "pivot",
             7: "convergence", 8: "no_device", 9: "handle", 10: "busy"}

EXPORTS = [
    "sspike_core_host", "dspike_core_host", "cspike_core_host", "zspike_core_host", "dspike_core_host_blocking",
    "SPIKE_SUCCESS", "SPIKE_ERROR", "spike_last_error_code", "spike_last_error", "spike_context_create",
    "spike_context_destroy", "spike_context_set_stream", "spike_set_option", "spike_get_option", "spike_get_info",
    "spike_dsolve_device", "spike_zsolve_device", "spike_dfactor", "spike_zfactor", "spike_dfactor_device",
    "spike_dsolve_factored", "spike_zsolve_factored", "spike_dsolve_factored_device", "spike_factor_release",
    "spike_get_phase_times", "spike_dsolve_device_noalloc", "spike_dbatch_create", "spike_batch_run",
    "spike_batch_relres", "spike_batch_get_info", "spike_batch_group", "spike_batch_destroy",
    "spike_batch_partitions", "spike_server_create", "spike_server_submit", "spike_server_wait",
    "spike_server_drain", "spike_server_stats", "spike_server_poll", "spike_server_clock", "spike_server_destroy",
    "spike_rcm_permutation", "spike_permute_csr", "spike_permute_vector", "spike_dsolve_reordered",
    "spike_csr_full_band", "spike_shard_range", "spike_shard_dsolve", "spike_shard_assemble", "spike_shard_split",
    "matrix_ComputeBandwidth", "matrix_LoadCSR", "matrix_SaveCSR", "matrix_ExportBinary",
    "matrix_CreateFromComponents", "matrix_Deallocate", "directSolver_CreateHandler", "directSolver_Configure",
    "directSolver_Factorize", "directSolver_SolveForRHS", "directSolver_ShowStatistics", "directSolver_Finalize",
    "spike_dsolve", "spike_zsolve", "directSolver_Solve", "block_CreateEmptyBlock", "block_Deallocate", "block_SaveCSR", "block_loadCSR",
    "vector_LoadPermutationArray", "vector_LoadRHS",
]
SPIKE_OPT_STREAM_ALLOC = 6
SPIKE_OPT_TWIST = 7
SPIKE_OPT_HOST_THREADS = 8
SPIKE_OPT_REDUCED_FP64 = 9
SPIKE_BATCH_AUTOTUNE = 1
SPIKE_BATCH_NO_GRAPH = 2


class SpikeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERR_NAMES.get(code, code)}] {msg}")
        self.code = code
        self.name = ERR_NAMES.get(code, str(code))


class Info(C.Structure):
    _fields_ = [("relres_max", C.c_double), ("refine_sweeps", C.c_int), ("partitions", C.c_int), ("ku", C.c_int),
                ("kl", C.c_int), ("block", C.c_int), ("kernel_launches", C.c_longlong),
                ("device_bytes", C.c_size_t), ("twisted", C.c_int), ("columns_implied", C.c_int),
                ("reduced_fp64", C.c_int)]


class DSystem(C.Structure):
    """spike_dsystem_t: one system of a batch (device pointers)."""
    _fields_ = [("n", C.c_int), ("nnz", C.c_int), ("nrhs", C.c_int), ("d_colind", C.c_void_p),
                ("d_rowptr", C.c_void_p), ("d_aij", C.c_void_p), ("d_x", C.c_void_p), ("d_b", C.c_void_p)]


class BatchInfo(C.Structure):
    _fields_ = [("systems", C.c_int), ("groups", C.c_int), ("graph", C.c_int), ("graph_sweeps", C.c_int),
                ("extra_sweeps", C.c_int), ("relres_max", C.c_double), ("graph_kernel_launches", C.c_longlong),
                ("device_bytes", C.c_size_t), ("tune_ms", C.c_double)]


class BatchGroup(C.Structure):
    _fields_ = [("block", C.c_int), ("nrhs", C.c_int), ("bandwidth", C.c_int), ("systems", C.c_int),
                ("partitions", C.c_int), ("rows_per_partition", C.c_int), ("graph_sweeps", C.c_int),
                ("rows", C.c_longlong), ("nnz", C.c_longlong)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("precision", C.c_int), ("tolerance", C.c_double), ("max_refine", C.c_int),
                ("hbm_budget", C.c_size_t), ("cache_budget", C.c_size_t), ("max_queue", C.c_int)]


class Request(C.Structure):
    _fields_ = [("n", C.c_int), ("nnz", C.c_int), ("nrhs", C.c_int), ("colind", C.c_void_p), ("rowptr", C.c_void_p),
                ("aij", C.c_void_p), ("b", C.c_void_p), ("x", C.c_void_p), ("bandwidth", C.c_int),
                ("factor_key", C.c_longlong), ("arrival", C.c_double)]


class RequestStatus(C.Structure):
    _fields_ = [("done", C.c_int), ("error_code", C.c_int), ("relres", C.c_double), ("sweeps", C.c_int),
                ("factor_hit", C.c_int), ("t_arrival", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("footprint", C.c_size_t)]


class Matrix(C.Structure):
    """matrix_t of the reference's double build (spike_compat.h)."""
    _fields_ = [("n", C.c_int), ("nnz", C.c_ulonglong), ("ku", C.c_int), ("kl", C.c_int), ("type", C.c_int),
                ("colind", C.POINTER(C.c_int)), ("rowptr", C.POINTER(C.c_int)), ("aij", C.POINTER(C.c_double))]


class Block(C.Structure):
    """block_t of the reference's double build (spike_compat.h)."""
    _fields_ = [("type", C.c_int), ("section", C.c_int), ("n", C.c_int), ("m", C.c_int), ("ku", C.c_int),
                ("kl", C.c_int), ("aij", C.POINTER(C.c_double))]


class DirectSolverHandler(C.Structure):
    """DirectSolverHander_t (spike_compat.h)."""
    _fields_ = [("ctx", C.c_void_p), ("factor", C.c_void_p), ("n", C.c_int), ("max_nrhs", C.c_int),
                ("factor_t", C.c_double), ("solve_t", C.c_double), ("rhs_block_count", C.c_int),
                ("rhs_column_count", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("rejected", C.c_longlong),
                ("failed", C.c_longlong), ("queued", C.c_longlong), ("factor_hits", C.c_longlong),
                ("factor_misses", C.c_longlong), ("running", C.c_int), ("peak_running", C.c_int),
                ("resident_factors", C.c_int), ("device_bytes_running", C.c_size_t),
                ("device_bytes_cached", C.c_size_t), ("latency_p50", C.c_double), ("latency_p99", C.c_double),
                ("latency_max", C.c_double), ("mean_queue_wait", C.c_double), ("throughput", C.c_double),
                ("relres_max", C.c_double), ("rejected_busy", C.c_longlong)]


_LIB = None
_GEN = None


def load(path: str | None = None):
    """Load libspike_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"native library missing: {path} (run hspike_gb300.build.build())")
    L = C.CDLL(path)
    ip, vp, i = C.POINTER(C.c_int), C.c_void_p, C.c_int
    for name in ("sspike_core_host", "dspike_core_host", "cspike_core_host", "zspike_core_host",
                 "dspike_core_host_blocking"):
        f = getattr(L, name)
        f.argtypes = [i, i, i, vp, vp, vp, vp, vp]
        f.restype = i
    L.spike_last_error_code.restype = i
    L.spike_last_error.restype = C.c_char_p
    L.spike_context_create.argtypes = [C.POINTER(vp)]
    L.spike_context_destroy.argtypes = [vp]
    L.spike_context_set_stream.argtypes = [vp, vp]
    L.spike_set_option.argtypes = [vp, i, C.c_double]
    L.spike_get_option.argtypes = [vp, i, C.POINTER(C.c_double)]
    L.spike_get_info.argtypes = [vp, C.POINTER(Info)]
    for name in ("spike_dsolve_device", "spike_zsolve_device", "spike_dsolve", "spike_zsolve"):
        getattr(L, name).argtypes = [vp, i, i, i, vp, vp, vp, vp, vp]
    for name in ("spike_dfactor", "spike_zfactor", "spike_dfactor_device"):
        getattr(L, name).argtypes = [vp, i, i, vp, vp, vp, C.POINTER(vp)]
    for name in ("spike_dsolve_factored", "spike_zsolve_factored", "spike_dsolve_factored_device"):
        getattr(L, name).argtypes = [vp, i, vp, vp]
    L.spike_factor_release.argtypes = [vp]
    L.spike_get_phase_times.argtypes = [vp, i, vp, vp, i]
    L.spike_dbatch_create.argtypes = [vp, i, vp, i, C.POINTER(vp)]
    L.spike_batch_run.argtypes = [vp]
    L.spike_batch_relres.argtypes = [vp, vp]
    L.spike_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    L.spike_batch_group.argtypes = [vp, i, C.POINTER(BatchGroup)]
    L.spike_batch_destroy.argtypes = [vp]
    L.spike_batch_partitions.argtypes = [i, i, i]
    L.spike_batch_partitions.restype = i
    L.spike_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(vp)]
    L.spike_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_longlong)]
    L.spike_server_wait.argtypes = [vp, C.c_longlong, C.POINTER(RequestStatus)]
    L.spike_server_poll.argtypes = [vp, C.c_longlong, C.POINTER(RequestStatus)]
    L.spike_server_drain.argtypes = [vp]
    L.spike_server_stats.argtypes = [vp, C.POINTER(ServerStats)]
    L.spike_server_clock.argtypes = [vp]
    L.spike_server_clock.restype = C.c_double
    L.spike_server_destroy.argtypes = [vp]
    L.spike_rcm_permutation.argtypes = [i, i, vp, vp, vp]
    L.spike_permute_csr.argtypes = [i, i, vp, vp, vp, vp, vp, vp, vp]
    L.spike_permute_vector.argtypes = [i, i, i, vp, vp]
    L.spike_dsolve_reordered.argtypes = [vp, i, i, i, vp, vp, vp, vp, vp, vp]
    L.spike_csr_full_band.argtypes = [i, i, i, i, vp, vp, C.POINTER(C.c_int)]
    L.spike_shard_range.argtypes = [i, i, i, i, ip, ip, ip, ip]
    L.spike_shard_dsolve.argtypes = [vp, vp, i, i, i, i, i, vp, vp, vp, vp, vp]
    L.spike_shard_assemble.argtypes = [i, i, i, i, vp, vp]
    L.spike_shard_split.argtypes = [i, i, i, i, vp, vp]
    mp, hp = C.POINTER(Matrix), C.POINTER(DirectSolverHandler)
    L.matrix_ComputeBandwidth.argtypes = [i, vp, vp, vp, ip, ip]
    L.matrix_LoadCSR.argtypes = [C.c_char_p]
    L.matrix_LoadCSR.restype = mp
    L.matrix_SaveCSR.argtypes = [C.c_char_p, mp]
    L.matrix_SaveCSR.restype = None
    L.matrix_ExportBinary.argtypes = [mp, C.c_char_p]
    L.matrix_CreateFromComponents.argtypes = [i, C.c_ulonglong, vp, vp, vp]
    L.matrix_CreateFromComponents.restype = mp
    L.matrix_Deallocate.argtypes = [mp]
    bp = C.POINTER(Block)
    L.block_CreateEmptyBlock.argtypes = [i, i, i, i, i, i]
    L.block_CreateEmptyBlock.restype = bp
    L.block_Deallocate.argtypes = [bp]
    L.block_SaveCSR.argtypes = [C.c_char_p, bp]
    L.block_SaveCSR.restype = None
    L.block_loadCSR.argtypes = [C.c_char_p]
    L.block_loadCSR.restype = bp
    L.vector_LoadPermutationArray.argtypes = [i, C.c_char_p]
    L.vector_LoadPermutationArray.restype = vp
    L.vector_LoadRHS.argtypes = [i, C.c_char_p]
    L.vector_LoadRHS.restype = vp
    L.directSolver_CreateHandler.argtypes = []
    L.directSolver_CreateHandler.restype = hp
    L.directSolver_Configure.argtypes = [hp, i]
    L.directSolver_Factorize.argtypes = [hp, i, i, vp, vp, vp]
    L.directSolver_SolveForRHS.argtypes = [hp, i, vp, vp]
    L.directSolver_ShowStatistics.argtypes = [hp]
    L.directSolver_Finalize.argtypes = [hp]
    L.directSolver_Solve.argtypes = [i, i, i, vp, vp, vp, vp, vp]
    _LIB = L
    return L


def last_error() -> tuple[int, str]:
    L = load()
    return L.spike_last_error_code(), (L.spike_last_error() or b"").decode()


def _check(rc: int):
    if rc != SPIKE_SUCCESS:
        code, msg = last_error()
        raise SpikeError(code, msg)


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


_DT = {"s": (np.float32, np.float32), "d": (np.float64, np.float64), "c": (np.complex64, np.complex64),
       "z": (np.complex128, np.complex128)}


def _core(prefix: str, n, nnz, nrhs, colind, rowptr, aij, x, b, blocking=False) -> int:
    """Call ``?spike_core_host`` with numpy arrays exactly like the C API.

    ``x`` is overwritten in place (column-major n x nrhs), as in the reference.
    """
    L = load()
    dt = _DT[prefix][0]
    for name, arr, want in (("colind", colind, np.int32), ("rowptr", rowptr, np.int32), ("aij", aij, dt),
                            ("x", x, dt), ("b", b, dt)):
        if arr.dtype != want:
            raise TypeError(f"{name} must be {np.dtype(want).name}, got {arr.dtype}")
        if not (arr.flags.f_contiguous or arr.flags.c_contiguous):
            raise ValueError(f"{name} must be contiguous")
    if x.ndim == 2 and not x.flags.f_contiguous:
        raise ValueError("x must be column-major (Fortran order)")
    fn = L.dspike_core_host_blocking if blocking else getattr(L, prefix + "spike_core_host")
    return fn(int(n), int(nnz), int(nrhs), _ptr(colind), _ptr(rowptr), _ptr(aij), _ptr(x), _ptr(b))


def sspike_core_host(n, nnz, nrhs, colind, rowptr, aij, x, b):
    return _core("s", n, nnz, nrhs, colind, rowptr, aij, x, b)


def dspike_core_host(n, nnz, nrhs, colind, rowptr, aij, x, b):
    return _core("d", n, nnz, nrhs, colind, rowptr, aij, x, b)


def cspike_core_host(n, nnz, nrhs, colind, rowptr, aij, x, b):
    return _core("c", n, nnz, nrhs, colind, rowptr, aij, x, b)


def zspike_core_host(n, nnz, nrhs, colind, rowptr, aij, x, b):
    return _core("z", n, nnz, nrhs, colind, rowptr, aij, x, b)


def dspike_core_host_blocking(n, nnz, nrhs, colind, rowptr, aij, x, b):
    return _core("d", n, nnz, nrhs, colind, rowptr, aij, x, b, blocking=True)


def set_option(option: int, value: float, ctx=None):
    _check(load().spike_set_option(ctx, option, float(value)))


def get_option(option: int, ctx=None) -> float:
    v = C.c_double()
    _check(load().spike_get_option(ctx, option, C.byref(v)))
    return v.value


def get_info(ctx=None) -> Info:
    info = Info()
    _check(load().spike_get_info(ctx, C.byref(info)))
    return info


def solve(rowptr, colind, aij, b, precision=SPIKE_PRECISION_MIXED, partitions=0, ctx=None):
    """x = A^{-1} b on the GPU through the C API; b may be 1-D or n x nrhs."""
    cplx = np.iscomplexobj(aij) or np.iscomplexobj(b)
    dt = np.complex128 if cplx else np.float64
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    aij = np.ascontiguousarray(aij, dt)
    b2 = np.asfortranarray(np.asarray(b, dt).reshape(len(rowptr) - 1, -1))
    x = np.zeros_like(b2, order="F")
    n, nrhs = b2.shape
    if ctx is not None:
        ctx.set_option(SPIKE_OPT_PRECISION, precision)
        ctx.set_option(SPIKE_OPT_PARTITIONS, partitions)
        fn = load().spike_zsolve if cplx else load().spike_dsolve
        rc = fn(ctx.handle, n, len(colind), nrhs, _ptr(colind), _ptr(rowptr), _ptr(aij), _ptr(x), _ptr(b2))
    else:
        set_option(SPIKE_OPT_PRECISION, precision)
        set_option(SPIKE_OPT_PARTITIONS, partitions)
        rc = _core("z" if cplx else "d", n, len(colind), nrhs, colind, rowptr, aij, x, b2)
    _check(rc)
    return x if np.ndim(b) == 2 else x[:, 0]


class Context:
    """An explicit solver context (own CUDA stream unless one is set)."""

    def __init__(self):
        self._h = C.c_void_p()
        _check(load().spike_context_create(C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle: int | None):
        _check(load().spike_context_set_stream(self._h, C.c_void_p(stream_handle or 0)))

    def set_option(self, option, value):
        set_option(option, value, self._h)

    def get_option(self, option):
        return get_option(option, self._h)

    def info(self) -> Info:
        return get_info(self._h)

    def phase_times(self, reset=True):
        """{family: (total ms, timed launches)} while SPIKE_OPT_PHASE_TIMING is on."""
        ms = np.zeros(len(PHASES), np.float64)
        calls = np.zeros(len(PHASES), np.int64)
        _check(load().spike_get_phase_times(self._h, len(PHASES), _ptr(ms), _ptr(calls), int(reset)))
        return {name: (float(ms[i]), int(calls[i])) for i, name in enumerate(PHASES)}

    def solve_device(self, n, nnz, nrhs, d_colind: int, d_rowptr: int, d_aij: int, d_x: int, d_b: int,
                     complex_=False):
        fn = load().spike_zsolve_device if complex_ else load().spike_dsolve_device
        _check(fn(self._h, n, nnz, nrhs, C.c_void_p(d_colind), C.c_void_p(d_rowptr), C.c_void_p(d_aij),
                  C.c_void_p(d_x), C.c_void_p(d_b)))

    def close(self):
        if self._h:
            load().spike_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Factor:
    """Factor once, solve many right-hand sides with resident factors."""

    def __init__(self, rowptr, colind, aij, ctx: Context | None = None):
        self.cplx = np.iscomplexobj(aij)
        dt = np.complex128 if self.cplx else np.float64
        self.rowptr = np.ascontiguousarray(rowptr, np.int32)
        self.colind = np.ascontiguousarray(colind, np.int32)
        self.aij = np.ascontiguousarray(aij, dt)
        self.n = len(self.rowptr) - 1
        self._h = C.c_void_p()
        fn = load().spike_zfactor if self.cplx else load().spike_dfactor
        _check(fn(ctx.handle if ctx else None, self.n, len(self.colind), _ptr(self.colind), _ptr(self.rowptr),
                  _ptr(self.aij), C.byref(self._h)))

    def solve(self, b):
        dt = np.complex128 if self.cplx else np.float64
        b2 = np.asfortranarray(np.asarray(b, dt).reshape(self.n, -1))
        x = np.zeros_like(b2, order="F")
        fn = load().spike_zsolve_factored if self.cplx else load().spike_dsolve_factored
        _check(fn(self._h, b2.shape[1], _ptr(x), _ptr(b2)))
        return x if np.ndim(b) == 2 else x[:, 0]

    def release(self):
        if self._h:
            _check(load().spike_factor_release(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class Batch:
    """Many independent systems (device arrays) solved by one graph launch.

    ``systems``: sequence of (n, nnz, nrhs, d_colind, d_rowptr, d_aij, d_x, d_b)
    with integer device addresses; x and b are n x nrhs column-major.
    """

    def __init__(self, systems, ctx: Context | None = None, autotune=True, graph=True):
        arr = (DSystem * len(systems))(*[DSystem(*s) for s in systems])
        flags = (SPIKE_BATCH_AUTOTUNE if autotune else 0) | (0 if graph else SPIKE_BATCH_NO_GRAPH)
        self.count = len(systems)
        self._h = C.c_void_p()
        _check(load().spike_dbatch_create(ctx.handle if ctx else None, len(systems), C.cast(arr, C.c_void_p), flags,
                                          C.byref(self._h)))

    def run(self):
        _check(load().spike_batch_run(self._h))

    def relres(self) -> np.ndarray:
        out = np.zeros(self.count, np.float64)
        _check(load().spike_batch_relres(self._h, _ptr(out)))
        return out

    def info(self) -> BatchInfo:
        inf = BatchInfo()
        _check(load().spike_batch_get_info(self._h, C.byref(inf)))
        return inf

    def groups(self) -> list[dict]:
        out = []
        for i in range(self.info().groups):
            g = BatchGroup()
            _check(load().spike_batch_group(self._h, i, C.byref(g)))
            out.append({f: getattr(g, f) for f, _ in BatchGroup._fields_})
        return out

    def destroy(self):
        if self._h:
            _check(load().spike_batch_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """The request loop of spike_server_*: ``slots`` concurrent requests,
    admission by device footprint, resident factors under keys."""

    def __init__(self, slots=4, precision=SPIKE_PRECISION_MIXED, tolerance=1e-12, max_refine=3, hbm_budget=0,
                 cache_budget=0, max_queue=0):
        cfg = ServerConfig(slots, precision, tolerance, max_refine, hbm_budget, cache_budget, max_queue)
        self._h = C.c_void_p()
        self._keep = {}
        _check(load().spike_server_create(C.byref(cfg), C.byref(self._h)))

    def submit(self, rowptr, colind, aij, b, x=None, factor_key=-1, bandwidth=-1, arrival=-1.0):
        """Queue A x = b (host arrays; x allocated if not given); returns (ticket, x)."""
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        colind = np.ascontiguousarray(colind, np.int32)
        aij = np.ascontiguousarray(aij, np.float64)
        n = len(rowptr) - 1
        b2 = np.asfortranarray(np.asarray(b, np.float64).reshape(n, -1))
        if x is None:
            x = np.zeros_like(b2, order="F")
        req = Request(n, len(colind), b2.shape[1], colind.ctypes.data, rowptr.ctypes.data, aij.ctypes.data,
                      b2.ctypes.data, x.ctypes.data, bandwidth, factor_key, arrival)
        t = C.c_longlong()
        _check(load().spike_server_submit(self._h, C.byref(req), C.byref(t)))
        self._keep[t.value] = (rowptr, colind, aij, b2, x)
        return t.value, x

    def wait(self, ticket, check=True) -> RequestStatus:
        st = RequestStatus()
        rc = load().spike_server_wait(self._h, ticket, C.byref(st))
        self._keep.pop(ticket, None)
        if check:
            _check(rc)
        return st

    def poll(self, ticket) -> RequestStatus:
        """The request's status now, without waiting; the arrays of a finished
        request are no longer held here (the caller keeps x)."""
        st = RequestStatus()
        _check(load().spike_server_poll(self._h, ticket, C.byref(st)))
        if st.done:
            self._keep.pop(ticket, None)
        return st

    def drain(self):
        _check(load().spike_server_drain(self._h))

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(load().spike_server_stats(self._h, C.byref(st)))
        return st

    def clock(self) -> float:
        return float(load().spike_server_clock(self._h))

    def close(self):
        if self._h:
            _check(load().spike_server_destroy(self._h))
            self._h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rcm_permutation(rowptr, colind) -> np.ndarray:
    """Reverse Cuthill-McKee order of the pattern of A + A^T (host, no device)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    n = len(rowptr) - 1
    perm = np.zeros(max(n, 1), np.int32)
    _check(load().spike_rcm_permutation(n, len(colind), _ptr(colind), _ptr(rowptr), _ptr(perm)))
    return perm[:n]


def permute_csr(rowptr, colind, aij, perm):
    """B = A(perm, perm) as (rowptr, colind, aij), rows sorted."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    aij = np.ascontiguousarray(aij, np.float64)
    perm = np.ascontiguousarray(perm, np.int32)
    n = len(rowptr) - 1
    orp, oci, oa = np.zeros(n + 1, np.int32), np.zeros(max(len(colind), 1), np.int32), np.zeros(max(len(aij), 1))
    _check(load().spike_permute_csr(n, len(colind), _ptr(colind), _ptr(rowptr), _ptr(aij), _ptr(perm), _ptr(oci),
                                    _ptr(orp), _ptr(oa)))
    return orp, oci[:len(colind)], oa[:len(aij)]


def permute_vector(flag, perm, v):
    """In place, column by column: flag > 0 -> v = v(perm); else v(perm) = v."""
    perm = np.ascontiguousarray(perm, np.int32)
    assert v.dtype == np.float64 and (v.flags.f_contiguous or v.ndim == 1)
    n = len(perm)
    _check(load().spike_permute_vector(flag, n, v.size // max(n, 1), _ptr(perm), _ptr(v)))
    return v


def solve_reordered(rowptr, colind, aij, b, ctx: Context | None = None):
    """x for a general sparse A: RCM + banded solve + back-permutation; returns (x, perm)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    aij = np.ascontiguousarray(aij, np.float64)
    n = len(rowptr) - 1
    b2 = np.asfortranarray(np.asarray(b, np.float64).reshape(n, -1))
    x = np.zeros_like(b2, order="F")
    perm = np.zeros(n, np.int32)
    _check(load().spike_dsolve_reordered(ctx.handle if ctx else None, n, len(colind), b2.shape[1], _ptr(colind),
                                         _ptr(rowptr), _ptr(aij), _ptr(x), _ptr(b2), _ptr(perm)))
    return (x if np.ndim(b) == 2 else x[:, 0]), perm


def batch_partitions(n: int, block: int, rows_per_partition: int) -> int:
    """The batch partition rule (host only, no device needed)."""
    return int(load().spike_batch_partitions(n, block, rows_per_partition))


def csr_full_band(rowptr, colind, ku: int, kl: int) -> bool:
    """True when every row r holds exactly the columns max(0, r - kl) ..
    min(n - 1, r + ku) in order: the layout whose column indices a solve with
    host arrays leaves on the host (host only, no device needed)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    full = C.c_int(-1)
    _check(load().spike_csr_full_band(len(rowptr) - 1, len(colind), ku, kl, _ptr(colind), _ptr(rowptr),
                                      C.byref(full)))
    return bool(full.value)


# ------------------------------------------------ reference matrix helpers + plugin
def compute_bandwidth(rowptr, colind) -> tuple[int, int]:
    """(ku, kl) by matrix_ComputeBandwidth (host)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    ku, kl = C.c_int(-1), C.c_int(-1)
    _check(load().matrix_ComputeBandwidth(len(rowptr) - 1, _ptr(colind), _ptr(rowptr), None, C.byref(ku),
                                          C.byref(kl)))
    return ku.value, kl.value


def load_csr(path: str):
    """matrix_LoadCSR: returns (rowptr, colind, aij, ku, kl) copied out of the matrix_t."""
    L = load()
    M = L.matrix_LoadCSR(os.fsencode(path))
    if not M:
        code, msg = last_error()
        raise SpikeError(code, msg)
    m = M.contents
    n, nnz = m.n, int(m.nnz)
    rowptr = np.ctypeslib.as_array(m.rowptr, (n + 1,)).copy()
    colind = np.ctypeslib.as_array(m.colind, (nnz,)).copy() if nnz else np.zeros(0, np.int32)
    aij = np.ctypeslib.as_array(m.aij, (nnz,)).copy() if nnz else np.zeros(0)
    ku, kl = m.ku, m.kl
    L.matrix_Deallocate(M)
    return rowptr, colind, aij, ku, kl


def save_csr(path: str, rowptr, colind, aij):
    """matrix_SaveCSR of a wrapping matrix_t (the arrays stay owned by numpy)."""
    L = load()
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    aij = np.ascontiguousarray(aij, np.float64)
    M = Matrix(len(rowptr) - 1, len(colind), 0, 0, 1, colind.ctypes.data_as(C.POINTER(C.c_int)),
               rowptr.ctypes.data_as(C.POINTER(C.c_int)), aij.ctypes.data_as(C.POINTER(C.c_double)))
    _check(L.matrix_ExportBinary(C.byref(M), os.fsencode(path)))


def save_block(path: str, a, ku=0, kl=0, type_=0, section=3):
    """block_SaveCSR of a dense column-major n x m block."""
    L = load()
    a = np.asfortranarray(np.asarray(a, np.float64).reshape(np.shape(a)[0], -1))
    B = L.block_CreateEmptyBlock(a.shape[0], a.shape[1], ku, kl, type_, section)
    if not B:
        code, msg = last_error()
        raise SpikeError(code, msg)
    C.memmove(B.contents.aij, a.ctypes.data, a.nbytes)
    L.block_SaveCSR(os.fsencode(path), B)
    code, msg = last_error()
    L.block_Deallocate(B)
    if code:
        raise SpikeError(code, msg)


def load_block(path: str):
    """block_loadCSR: returns (aij n x m column-major, type, section, ku, kl)."""
    L = load()
    B = L.block_loadCSR(os.fsencode(path))
    if not B:
        code, msg = last_error()
        raise SpikeError(code, msg)
    b = B.contents
    a = np.ctypeslib.as_array(b.aij, (b.n * b.m,)).copy() if b.n * b.m else np.zeros(0)
    out = (a.reshape((b.n, b.m), order="F"), b.type, b.section, b.ku, b.kl)
    L.block_Deallocate(B)
    return out


def load_vector(path: str, n: int, permutation=False):
    """vector_LoadPermutationArray (int32) or vector_LoadRHS (float64): n raw entries."""
    L = load()
    f = L.vector_LoadPermutationArray if permutation else L.vector_LoadRHS
    p = f(n, os.fsencode(path))
    if not p:
        code, msg = last_error()
        raise SpikeError(code, msg)
    ct = C.c_int if permutation else C.c_double
    v = np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), (n,)).copy() if n else np.zeros(0, ct)
    C.CDLL(None).free(C.c_void_p(p))
    return v


class DirectSolver:
    """The directSolver_* plugin: factor once on the device, solve many times."""

    def __init__(self, max_nrhs: int | None = None):
        self.L = load()
        self.h = self.L.directSolver_CreateHandler()
        if not self.h:
            code, msg = last_error()
            raise SpikeError(code, msg)
        if max_nrhs is not None:
            _check(self.L.directSolver_Configure(self.h, max_nrhs))

    def factorize(self, rowptr, colind, aij):
        self._keep = (np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colind, np.int32),
                      np.ascontiguousarray(aij, np.float64))
        rp, ci, a = self._keep
        _check(self.L.directSolver_Factorize(self.h, len(rp) - 1, len(ci), _ptr(ci), _ptr(rp), _ptr(a)))

    def solve(self, b):
        b = np.asarray(b, np.float64)
        b2 = np.asfortranarray(b.reshape(self.h.contents.n or len(b), -1))
        x = np.zeros_like(b2, order="F")
        _check(self.L.directSolver_SolveForRHS(self.h, b2.shape[1], _ptr(x), _ptr(b2)))
        return x if np.ndim(b) == 2 else x[:, 0]

    @property
    def stats(self) -> DirectSolverHandler:
        return self.h.contents

    def close(self):
        if self.h:
            _check(self.L.directSolver_Finalize(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def direct_solve(rowptr, colind, aij, b):
    """directSolver_Solve: factor + solve + release in one call."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    aij = np.ascontiguousarray(aij, np.float64)
    n = len(rowptr) - 1
    b2 = np.asfortranarray(np.asarray(b, np.float64).reshape(n, -1))
    x = np.zeros_like(b2, order="F")
    _check(load().directSolver_Solve(n, len(colind), b2.shape[1], _ptr(colind), _ptr(rowptr), _ptr(aij), _ptr(x),
                                     _ptr(b2)))
    return x if np.ndim(b) == 2 else x[:, 0]


# ---------------------------------------------------------------- generator
def _gen():
    global _GEN
    if _GEN is None:
        path = gen_path()
        if not os.path.exists(path):
            raise RuntimeError(f"generator library missing: {path} (run hspike_gb300.build.build())")
        G = C.CDLL(path)
        G.spike_gen_rowptr.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p]
        G.spike_gen_rowptr.restype = C.c_longlong
        G.spike_gen_fill.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_ulonglong, C.c_int, C.c_int,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        G.spike_gen_fill.restype = C.c_int
        _GEN = G
    return _GEN


def gen_banded(n, ku, kl, dom, seed, complex_=False, nrhs=1, alloc=None):
    """Seeded banded system: returns (rowptr, colind, aij, x_true, b).

    Off-diagonals U[-1,1) (re/im i.i.d. for complex); diagonal = dom * (sum of
    the row's off-diagonal magnitudes) * (random sign, or e^{i theta});
    x_true U[-1,1); b = A x_true in double.  ``alloc(shape, dtype)`` may supply
    the arrays (e.g. pinned host memory); it defaults to numpy.empty.
    """
    G = _gen()
    alloc = alloc or (lambda shape, dtype: np.empty(shape, dtype))
    rowptr = alloc((n + 1,), np.int32)
    nnz = int(G.spike_gen_rowptr(n, ku, kl, _ptr(rowptr)))
    colind = alloc((nnz,), np.int32)
    dt = np.complex128 if complex_ else np.float64
    aij = alloc((nnz,), dt)
    x_true = alloc((n * nrhs,), dt)
    b = alloc((n * nrhs,), dt)
    G.spike_gen_fill(n, ku, kl, float(dom), int(seed), 1 if complex_ else 0, nrhs, _ptr(rowptr), _ptr(colind),
                     _ptr(aij), _ptr(x_true), _ptr(b))
    x_true = x_true.reshape((n, nrhs), order="F")
    b = b.reshape((n, nrhs), order="F")
    return rowptr, colind, aij, x_true, b
