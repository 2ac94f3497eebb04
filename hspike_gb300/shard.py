"""One SPIKE solve sharded across ranks (processes, one GPU each).

ctypes mirror of the ``spike_shard_*`` entry points of
``include/spike_gb300.h`` -- the replacement for the reference's MPI
master/worker solve (MPI/spike_dm.c:21-202) -- and ``TorchComm``, a
``spike_comm_t`` whose callbacks run over a ``torch.distributed`` process
group on host buffers (gloo, or any backend that takes CPU tensors).

    comm = TorchComm()                       # after dist.init_process_group
    part0, part1, row0, row1 = shard_range(n, p, comm.size, comm.rank)
    x_rows = shard_solve(comm, n, p, rowptr_rows, colind_rows, aij_rows, b_rows)

Every rank passes the CSR rows [row0, row1) (row pointers rebased to 0,
GLOBAL column indices) and those rows of b, and gets the same rows of x.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _check, load

GATHER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p)
SCATTER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p)
ALLREDUCE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_int)
EXCHANGE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t)


class Comm(C.Structure):
    """spike_comm_t"""
    _fields_ = [("rank", C.c_int), ("size", C.c_int), ("user", C.c_void_p), ("gather", GATHER),
                ("scatter", SCATTER), ("allreduce_sum", ALLREDUCE), ("exchange", EXCHANGE)]


def _bytes_at(ptr: int, nbytes: int) -> np.ndarray:
    return np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(ptr)) if nbytes else np.zeros(0, np.uint8)


class TorchComm:
    """spike_comm_t over a torch.distributed group: gather / scatter to and
    from rank 0 of the group, an all-reduce sum, and point-to-point sends to
    the neighbouring ranks.  A callback that raises reports failure (1) to the
    library, which then returns SPIKE_ERROR."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist

        self.torch, self.dist, self.group = torch, dist, group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        self._root = dist.get_global_rank(group, 0) if group is not None else 0
        self._cbs = (GATHER(self._gather), SCATTER(self._scatter), ALLREDUCE(self._allreduce),
                     EXCHANGE(self._exchange))  # kept alive with the object
        self.c = Comm(self.rank, self.size, None, *self._cbs)

    def _peer(self, r):
        return self.dist.get_global_rank(self.group, r) if self.group is not None else r

    def _t(self, ptr, nbytes):
        return self.torch.from_numpy(_bytes_at(ptr, nbytes))

    def _gather(self, user, send, nbytes, recv):
        try:
            t = self._t(send, nbytes)
            if self.rank == 0:  # each rank's part lands in its slot of recv
                dst = _bytes_at(recv, nbytes * self.size)
                out = [self.torch.from_numpy(dst[r * nbytes:(r + 1) * nbytes]) for r in range(self.size)]
                self.dist.gather(t, out, dst=self._root, group=self.group)
            else:
                self.dist.gather(t, None, dst=self._root, group=self.group)
            return 0
        except Exception:  # noqa: BLE001 -- reported to the library as a failed transfer
            return 1

    def _scatter(self, user, send, nbytes, recv):
        try:
            t = self._t(recv, nbytes)
            if self.rank == 0:
                src = _bytes_at(send, nbytes * self.size)
                parts = [self.torch.from_numpy(src[r * nbytes:(r + 1) * nbytes]) for r in range(self.size)]
                self.dist.scatter(t, parts, src=self._root, group=self.group)
            else:
                self.dist.scatter(t, None, src=self._root, group=self.group)
            return 0
        except Exception:  # noqa: BLE001
            return 1

    def _allreduce(self, user, buf, count):
        try:
            arr = np.ctypeslib.as_array(buf, shape=(count,))
            self.dist.all_reduce(self.torch.from_numpy(arr), group=self.group)
            return 0
        except Exception:  # noqa: BLE001
            return 1

    def _exchange(self, user, to_lo, to_hi, from_lo, from_hi, nbytes):
        try:
            reqs = []
            if self.rank > 0:
                reqs.append(self.dist.isend(self._t(to_lo, nbytes).clone(), self._peer(self.rank - 1), group=self.group))
                reqs.append(self.dist.irecv(self._t(from_lo, nbytes), self._peer(self.rank - 1), group=self.group))
            if self.rank < self.size - 1:
                reqs.append(self.dist.isend(self._t(to_hi, nbytes).clone(), self._peer(self.rank + 1), group=self.group))
                reqs.append(self.dist.irecv(self._t(from_hi, nbytes), self._peer(self.rank + 1), group=self.group))
            for r in reqs:
                r.wait()
            return 0
        except Exception:  # noqa: BLE001
            return 1


def shard_range(n: int, p: int, size: int, rank: int) -> tuple[int, int, int, int]:
    """(part0, part1, row0, row1) of rank `rank` of `size` (spike_shard_range)."""
    out = [C.c_int() for _ in range(4)]
    _check(load().spike_shard_range(n, p, size, rank, *[C.byref(o) for o in out]))
    return tuple(o.value for o in out)


def slot_records(p: int, size: int) -> int:
    """records per rank slot in spike_shard_assemble / spike_shard_split"""
    return -(-p // size) + 1


def assemble(p: int, size: int, left_len: int, right_len: int, slots: np.ndarray) -> np.ndarray:
    """The p - 1 global records from every rank's slot (spike_shard_assemble)."""
    slots = np.ascontiguousarray(slots, np.float64)
    out = np.zeros((p - 1) * (left_len + right_len), np.float64)
    _check(load().spike_shard_assemble(p, size, left_len, right_len, slots.ctypes.data, out.ctypes.data))
    return out


def split(p: int, size: int, left_len: int, right_len: int, glob: np.ndarray) -> np.ndarray:
    """Every rank's slot from the global records (spike_shard_split)."""
    glob = np.ascontiguousarray(glob, np.float64)
    out = np.zeros(size * slot_records(p, size) * (left_len + right_len), np.float64)
    _check(load().spike_shard_split(p, size, left_len, right_len, glob.ctypes.data, out.ctypes.data))
    return out


def shard_solve(comm: TorchComm, n: int, p: int, rowptr, colind, aij, b, ctx=None) -> np.ndarray:
    """This rank's rows of x = A^{-1} b, solved by every rank of `comm` together
    (spike_shard_dsolve); b: this rank's rows, 1-D or rows x nrhs."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colind = np.ascontiguousarray(colind, np.int32)
    aij = np.ascontiguousarray(aij, np.float64)
    b2 = np.asfortranarray(np.asarray(b, np.float64).reshape(len(rowptr) - 1, -1))
    x = np.zeros_like(b2, order="F")
    rows, nrhs = b2.shape
    handle = ctx.handle if ctx is not None else None
    _check(load().spike_shard_dsolve(handle, C.byref(comm.c), n, p, nrhs, rows, len(colind), colind.ctypes.data,
                                     rowptr.ctypes.data, aij.ctypes.data, x.ctypes.data, b2.ctypes.data))
    return x if np.ndim(b) == 2 else x[:, 0]


def rows_of(rowptr, colind, aij, row0: int, row1: int):
    """The CSR rows [row0, row1) of a whole matrix, row pointers rebased to 0
    (what one rank holds)."""
    t0, t1 = int(rowptr[row0]), int(rowptr[row1])
    return (np.asarray(rowptr[row0:row1 + 1], np.int64) - t0).astype(np.int32), colind[t0:t1], aij[t0:t1]
