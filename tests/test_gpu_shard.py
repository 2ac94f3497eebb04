"""The sharded solve (spike_shard_dsolve) on the GPU: 2 and 3 ranks.

Each rank is a process with its own CUDA context on the same GPU and a gloo
group for the exchanges (TorchComm: tips gathered to rank 0, interface
unknowns scattered back, x halos with the neighbours, norms summed); no
kernel of one rank waits on another's.  Each rank passes only its rows of A
and b.  The assembled x is held to the parity bar against the CPU oracle
(oracle/spike_oracle.c, the restated reference path) with the same p, and
against the single-GPU solve:

    relative residual <= 1e-12,   ||x - x_oracle|| / ||x_oracle|| <= 1e-9

The reference's distributed variant is MPI/spike_dm.c:21-202.
"""
import socket

import numpy as np
import pytest

import hspike_gb300 as hs
from hspike_gb300 import shard

pytestmark = pytest.mark.gpu

RES_TOL = 1e-12
ERR_TOL = 1e-9


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, size, port, case, outq):
    try:
        import torch
        import torch.distributed as dist

        n, k, p, nrhs, prec, seed = case
        torch.cuda.set_device(0)
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=size)
        comm = shard.TorchComm()
        rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed, nrhs=nrhs)
        part0, part1, row0, row1 = shard.shard_range(n, p, size, rank)
        lrp, lci, la = shard.rows_of(rp, ci, a, row0, row1)
        ctx = hs.Context()
        ctx.set_option(hs.SPIKE_OPT_PRECISION, prec)
        x = shard.shard_solve(comm, n, p, lrp, lci, la, b[row0:row1], ctx=ctx)
        info = ctx.info()
        outq.put((rank, row0, row1, x, info.relres_max, info.refine_sweeps, info.twisted))
        ctx.close()
        dist.destroy_process_group()
    except BaseException as e:  # noqa: BLE001 -- reported to the parent
        outq.put((rank, None, None, f"{type(e).__name__}: {e}", None, None, None))
        raise


def _run(size, case):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, size, port, case, q)) for r in range(size)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=600) for _ in range(size)]
    for pr in procs:
        pr.join(timeout=120)
    for pr in procs:
        if pr.is_alive():
            pr.kill()
    errs = [r for r in res if r[1] is None]
    assert not errs, errs
    assert all(pr.exitcode == 0 for pr in procs)
    return sorted(res)


CASES = [  # n, k, p, nrhs, precision, seed
    (40_000, 8, 16, 2, hs.SPIKE_PRECISION_MIXED, 11),
    (130_000, 64, 32, 1, hs.SPIKE_PRECISION_MIXED, 12),
    (30_000, 3, 12, 3, hs.SPIKE_PRECISION_FP64, 13),
]


@pytest.mark.parametrize("size", [2, 3])
@pytest.mark.parametrize("case", CASES)
def test_sharded_solve_matches_the_oracle_and_one_gpu(size, case):
    from oracle import oracle

    n, k, p, nrhs, prec, seed = case
    res = _run(size, case)
    x = np.zeros((n, nrhs))
    for rank, r0, r1, xr, relres, sweeps, twisted in res:
        x[r0:r1] = xr.reshape(r1 - r0, nrhs)
    # every rank reports the same global relative residual and sweep count
    assert len({r[4] for r in res}) == 1 and len({r[5] for r in res}) == 1
    assert res[0][4] <= RES_TOL
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed, nrhs=nrhs)
    assert oracle.residual(rp, ci, a, x, b).max() <= RES_TOL
    xo = oracle.spike(rp, ci, a, b, p=p)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= ERR_TOL
    x1 = hs.solve(rp, ci, a, b, precision=prec, partitions=p)
    assert np.linalg.norm(x - x1) / np.linalg.norm(x1) <= ERR_TOL
    if k == 64:
        assert all(r[6] == 1 for r in res)  # the ranks' partitions were eliminated from both ends


def _rank_sequence(rank, size, port, outq):
    """One context through a sequence of sharded solves: the same system twice
    (the plans and buffers kept from the first call), a different shape, a
    wider band (a larger tile), a call with an out-of-range column on rank 1
    only (every rank gets an error, nothing is kept), then the first system
    again."""
    try:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(0)
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=size)
        comm = shard.TorchComm()
        ctx = hs.Context()
        out = []

        def one(n, k, p, seed, corrupt=False):
            rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed, nrhs=1)
            part0, part1, row0, row1 = shard.shard_range(n, p, size, rank)
            lrp, lci, la = shard.rows_of(rp, ci, a, row0, row1)
            if corrupt and rank == 1:
                lci = lci.copy()
                lci[len(lci) // 2] = n + 5
            try:
                x = shard.shard_solve(comm, n, p, lrp, lci, la, b[row0:row1], ctx=ctx)
            except hs.SpikeError as e:
                out.append(("error", e.code))
                return
            xr = np.asarray(xt).reshape(n, -1)[row0:row1, 0]
            err = float(np.linalg.norm(x.ravel() - xr) / np.linalg.norm(xr))
            out.append(("ok", ctx.info().block, ctx.info().relres_max, err))

        one(40_000, 8, 16, 21)
        one(40_000, 8, 16, 21)
        one(52_000, 8, 20, 22)
        one(52_000, 40, 20, 23)
        one(52_000, 40, 20, 23, corrupt=True)
        one(40_000, 8, 16, 21)
        outq.put((rank, out))
        ctx.close()
        dist.destroy_process_group()
    except BaseException as e:  # noqa: BLE001 -- reported to the parent
        outq.put((rank, f"{type(e).__name__}: {e}"))
        raise


def test_sharded_solves_in_sequence_on_one_context():
    import multiprocessing as mp

    size = 2
    mpc = mp.get_context("spawn")
    q = mpc.Queue()
    port = _free_port()
    procs = [mpc.Process(target=_rank_sequence, args=(r, size, port, q)) for r in range(size)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=600) for _ in range(size))
    for pr in procs:
        pr.join(timeout=120)
    for pr in procs:
        if pr.is_alive():
            pr.kill()
    assert all(isinstance(r[1], list) for r in res), res
    for rank, out in res:
        ok = [o for o in out if o[0] == "ok"]
        assert [o[1] for o in ok] == [8, 8, 8, 64, 8]  # tile size of each successful call
        assert all(o[2] <= RES_TOL and o[3] <= 1e-10 for o in ok), out
        assert out[4][0] == "error"
    # the rank with the bad column reports it; the other learns that a peer failed
    assert res[1][1][4][1] == 2  # SPIKE_ERR_CSR-class code on rank 1
    assert res[0][1][4][1] != 0
    for rank, out in res:  # same system, same x each time (the norms' float atomics may move relres's last bits)
        assert out[0][3] == out[1][3] == out[5][3]
        assert out[1][2] == pytest.approx(out[0][2], rel=1e-6) and out[5][2] == pytest.approx(out[0][2], rel=1e-6)
