"""Host side of the sharded solve, without a GPU.

* spike_shard_range: contiguous ranges that tile every partition and row,
  with the reference's partition boundaries (OpenMP/spike_analysis.c:38-76);
* spike_shard_assemble / spike_shard_split: the routing of the reduced
  system's records between ranks -- each half of a boundary interface comes
  from the rank that owns its partition (the tips gathered by the master in
  MPI/spike_mpi.c:450-674);
* the same routing over a real two-rank gloo group (TorchComm's gather,
  scatter, all-reduce and neighbour exchange), as spike_shard_dsolve uses it.
"""
import os
import socket

import numpy as np
import pytest

from hspike_gb300 import shard


@pytest.mark.parametrize("n,p,size", [(1000, 4, 1), (1000, 4, 2), (1003, 7, 3), (100_000, 256, 8), (57, 5, 5)])
def test_ranges_tile_rows_and_partitions(n, p, size):
    parts, rows = [], []
    for r in range(size):
        a, b, r0, r1 = shard.shard_range(n, p, size, r)
        parts.append((a, b))
        rows.append((r0, r1))
        assert r0 == a * (n // p) and r1 == (b * (n // p) if b < p else n)
        assert (b - a) in (p // size, -(-p // size))  # balanced to within one partition
    assert parts[0][0] == 0 and parts[-1][1] == p and rows[0][0] == 0 and rows[-1][1] == n
    for (a0, b0), (a1, b1) in zip(parts, parts[1:]):
        assert b0 == a1
    for (r0, r1), (s0, s1) in zip(rows, rows[1:]):
        assert r1 == s0


def test_range_rejects_bad_arguments():
    import hspike_gb300 as hs
    with pytest.raises(hs.SpikeError):
        shard.shard_range(100, 4, 5, 0)  # more ranks than partitions
    with pytest.raises(hs.SpikeError):
        shard.shard_range(100, 4, 2, 2)


def _slots_from(glob, p, size, L, R, rng):
    """What each rank would produce: its local interfaces' records, the halves
    it does not own (the neighbours' partitions) filled with noise."""
    rec = L + R
    nrec = shard.slot_records(p, size)
    slots = rng.standard_normal(size * nrec * rec)
    for r in range(size):
        a, b, _, _ = shard.shard_range(10 * p, p, size, r)
        for j in range(b - a + 1):
            g = a - 1 + j
            if 0 <= g <= p - 2:
                dst = slots[(r * nrec + j) * rec:(r * nrec + j + 1) * rec]
                if j > 0:
                    dst[:L] = glob[g * rec:g * rec + L]
                if j < b - a:
                    dst[L:] = glob[g * rec + L:(g + 1) * rec]
    return slots


@pytest.mark.parametrize("p,size", [(2, 1), (2, 2), (9, 2), (9, 4), (16, 3), (5, 5)])
def test_assemble_takes_each_half_from_its_owner_and_split_returns_whole_records(p, size):
    rng = np.random.default_rng(p * 10 + size)
    L, R = 6, 4
    glob = rng.standard_normal((p - 1) * (L + R))
    slots = _slots_from(glob, p, size, L, R, rng)
    np.testing.assert_array_equal(shard.assemble(p, size, L, R, slots), glob)
    back = shard.split(p, size, L, R, glob).reshape(size, shard.slot_records(p, size), L + R)
    for r in range(size):
        a, b, _, _ = shard.shard_range(10 * p, p, size, r)
        for j in range(back.shape[1]):
            g = a - 1 + j
            want = glob[g * (L + R):(g + 1) * (L + R)] if (j <= b - a and 0 <= g <= p - 2) else np.zeros(L + R)
            np.testing.assert_array_equal(back[r, j], want)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _routing_rank(rank, size, port, p, errq):
    try:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=size)
        comm = shard.TorchComm()
        assert (comm.rank, comm.size) == (rank, size)
        rng = np.random.default_rng(77)  # the same global records on every rank
        L, R = 5, 3
        glob = rng.standard_normal((p - 1) * (L + R))
        slots = _slots_from(glob, p, size, L, R, np.random.default_rng(5))
        nrec = shard.slot_records(p, size)
        slot_len = nrec * (L + R)
        mine = np.ascontiguousarray(slots[rank * slot_len:(rank + 1) * slot_len])
        allslots = np.zeros(size * slot_len) if rank == 0 else np.zeros(1)
        assert comm._gather(None, mine.ctypes.data, mine.nbytes, allslots.ctypes.data) == 0
        if rank == 0:
            np.testing.assert_array_equal(shard.assemble(p, size, L, R, allslots), glob)
            out = shard.split(p, size, L, R, glob)
        else:
            out = np.zeros(1)
        got = np.zeros(slot_len)
        assert comm._scatter(None, out.ctypes.data, got.nbytes, got.ctypes.data) == 0
        want = shard.split(p, size, L, R, glob)[rank * slot_len:(rank + 1) * slot_len]
        np.testing.assert_array_equal(got, want)
        # all-reduce sum in place
        v = np.array([rank + 1.0, 2.0 * rank], np.float64)
        assert comm._allreduce(None, v.ctypes.data_as(shard.C.POINTER(shard.C.c_double)), 2) == 0
        np.testing.assert_array_equal(v, [sum(r + 1.0 for r in range(size)), sum(2.0 * r for r in range(size))])
        # neighbour exchange: rank r sends (r, lo) down and (r, hi) up
        to_lo, to_hi = np.full(4, 10.0 * rank + 1), np.full(4, 10.0 * rank + 2)
        from_lo, from_hi = np.full(4, -1.0), np.full(4, -1.0)
        assert comm._exchange(None, to_lo.ctypes.data, to_hi.ctypes.data, from_lo.ctypes.data, from_hi.ctypes.data,
                              to_lo.nbytes) == 0
        if rank > 0:
            np.testing.assert_array_equal(from_lo, np.full(4, 10.0 * (rank - 1) + 2))
        if rank < size - 1:
            np.testing.assert_array_equal(from_hi, np.full(4, 10.0 * (rank + 1) + 1))
        dist.destroy_process_group()
    except BaseException as e:  # noqa: BLE001 -- reported to the parent
        errq.put(f"rank {rank}: {type(e).__name__}: {e}")
        raise


@pytest.mark.parametrize("size,p", [(2, 7), (3, 9)])
def test_routing_over_a_gloo_group(size, p):
    pytest.importorskip("torch")
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    errq = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_routing_rank, args=(r, size, port, p, errq)) for r in range(size)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=240)
    alive = [pr for pr in procs if pr.is_alive()]
    for pr in alive:
        pr.kill()
    errs = []
    while not errq.empty():
        errs.append(errq.get())
    assert not alive, "a rank did not finish"
    assert not errs and all(pr.exitcode == 0 for pr in procs), errs
