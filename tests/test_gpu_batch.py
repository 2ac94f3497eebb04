"""Batched solve of many independent systems (spike_dbatch_create / spike_batch_run).

Each system of a batch must come out as it does alone: the same solution as
the single-system device entry point (relative difference <= 1e-9), and a
relative residual <= 1e-12 against the oracle's FP64 residual.  Covers
uneven n, bandwidth and nrhs in one batch, systems shorter than two tiles,
graph replay with new values of b, the eager path, both precisions and the
autotuner.
"""
import numpy as np
import pytest

import hspike_gb300 as hs
from hspike_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-9
RES_TOL = 1e-12


def _device_batch(hb, torch, dev):
    t = {k: torch.from_numpy(getattr(hb, k)).to(dev) for k in ("rowptr", "colind", "aij", "b")}
    t["x"] = torch.zeros_like(t["b"])
    systems = []
    for i, (n, k, nrhs, _) in enumerate(hb.draws):
        nnz = W.nnz_banded(n, k, k)
        systems.append((n, nnz, nrhs, t["colind"].data_ptr() + 4 * int(hb.nz_off[i]),
                        t["rowptr"].data_ptr() + 4 * int(hb.rp_off[i]), t["aij"].data_ptr() + 8 * int(hb.nz_off[i]),
                        t["x"].data_ptr() + 8 * int(hb.v_off[i]), t["b"].data_ptr() + 8 * int(hb.v_off[i])))
    return t, systems


def _x_of(hb, t, i):
    n, k, nrhs, _ = hb.draws[i]
    o = int(hb.v_off[i])
    return t["x"][o:o + n * nrhs].cpu().numpy().reshape((n, nrhs), order="F")


def _check_against_single(hb, t, torch, dev, precision, idx):
    from oracle import oracle
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PRECISION, precision)
    for i in idx:
        rp, ci, a, xt, b = hb.system(i)
        n, k, nrhs, _ = hb.draws[i]
        x = _x_of(hb, t, i)
        assert np.isfinite(x).all(), i
        res = oracle.residual(rp, ci, a, x, b).max()
        assert res <= RES_TOL, (i, hb.draws[i], res)
        # the same system through the single-system device entry point
        d_rp, d_ci, d_a = (torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in (rp, ci, a))
        d_b = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev)
        d_x = torch.zeros_like(d_b)
        ctx.solve_device(n, len(ci), nrhs, d_ci.data_ptr(), d_rp.data_ptr(), d_a.data_ptr(), d_x.data_ptr(),
                         d_b.data_ptr())
        torch.cuda.synchronize()
        ref = d_x.cpu().numpy().T
        err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
        assert err <= ERR_TOL, (i, hb.draws[i], err)
        assert np.linalg.norm(x - xt) / np.linalg.norm(xt) <= 1e-9, i
    ctx.close()


@pytest.mark.parametrize("precision", [hs.SPIKE_PRECISION_MIXED, hs.SPIKE_PRECISION_FP64])
def test_batch_matches_single_solves(precision):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    draws = W.batch_draws(40, seed=11, n_range=(300, 6000))
    draws.append((40, 32, 4, 1.5))   # shorter than two tiles: one partition, no distinct tips
    draws.append((70, 8, 1, 1.3))
    draws.append((20, 32, 1, 1.5))   # shorter than one tile (band clipped to n - 1 = 19)
    draws.append((5000, 0, 2, 1.5))  # diagonal
    if precision == hs.SPIKE_PRECISION_MIXED:  # 128-row tiles (real mixed precision only)
        draws += [(3000, 100, 2, 1.5), (9000, 128, 1, 1.3), (200, 90, 1, 1.5)]
    hb = W.gen_batch(draws, seed=11)
    t, systems = _device_batch(hb, torch, dev)
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PRECISION, precision)
    bt = hs.Batch(systems, ctx, autotune=False)
    bt.run()
    info = bt.info()
    assert info.graph == 1 and info.groups >= 5 and info.relres_max <= RES_TOL
    rr = bt.relres()
    assert (rr <= RES_TOL).all()
    groups = bt.groups()
    assert sum(g["systems"] for g in groups) == len(draws)
    for g in groups:  # partitions never straddle systems: at least one per system
        assert g["partitions"] >= g["systems"]
    _check_against_single(hb, t, torch, dev, precision, range(len(draws)))
    bt.destroy()
    ctx.close()


def test_batch_graph_replay_reads_new_values():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    draws = W.batch_draws(24, seed=12, n_range=(500, 4000))
    hb = W.gen_batch(draws, seed=12)
    t, systems = _device_batch(hb, torch, dev)
    bt = hs.Batch(systems, autotune=False)
    bt.run()
    x1 = [_x_of(hb, t, i).copy() for i in range(len(draws))]
    # new right-hand sides and a rescaled matrix, same pointers: one more graph replay
    rng = np.random.default_rng(3)
    newb = rng.standard_normal(hb.b.shape)
    t["b"].copy_(torch.from_numpy(newb))
    t["aij"].mul_(2.0)
    bt.run()
    from oracle import oracle
    for i in range(len(draws)):
        rp, ci, a, xt, b = hb.system(i)
        n, k, nrhs, _ = draws[i]
        o = int(hb.v_off[i])
        b2 = newb[o:o + n * nrhs].reshape((n, nrhs), order="F")
        x = _x_of(hb, t, i)
        assert oracle.residual(rp, ci, 2.0 * a, x, b2).max() <= RES_TOL, i
        assert not np.allclose(x, x1[i])
    bt.destroy()


def test_batch_eager_and_autotuned_agree():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    draws = W.batch_draws(30, seed=13, n_range=(1000, 8000))
    hb = W.gen_batch(draws, seed=13)
    t, systems = _device_batch(hb, torch, dev)
    eager = hs.Batch(systems, autotune=False, graph=False)
    eager.run()
    assert eager.info().graph == 0
    xs = [_x_of(hb, t, i).copy() for i in range(len(draws))]
    t["x"].zero_()
    tuned = hs.Batch(systems, autotune=True)
    assert tuned.info().tune_ms > 0
    tuned.run()
    for i in range(len(draws)):
        x = _x_of(hb, t, i)
        assert np.linalg.norm(x - xs[i]) / np.linalg.norm(xs[i]) <= ERR_TOL, i
    assert (tuned.relres() <= RES_TOL).all()
    eager.destroy()
    tuned.destroy()


def test_batch_band_above_fp64_tiles_is_rejected():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    hb = W.gen_batch([(1000, 2, 1, 1.5), (2000, 100, 1, 1.5)], seed=15)
    t, systems = _device_batch(hb, torch, dev)
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_FP64)
    with pytest.raises(hs.SpikeError) as e:
        hs.Batch(systems, ctx, autotune=False)
    assert e.value.name == "bandwidth" and "system 1" in str(e.value)
    ctx.close()


def test_handles_outlive_their_context():
    # a factor handle and a batch released after their context is destroyed
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rp, ci, a, xt, b = hs.gen_banded(20000, 8, 8, 1.5, seed=91)
    ctx = hs.Context()
    f = hs.Factor(rp, ci, a, ctx)
    hb = W.gen_batch([(3000, 3, 1, 1.5), (5000, 8, 2, 1.5)], seed=92)
    t, systems = _device_batch(hb, torch, dev)
    bt = hs.Batch(systems, ctx, autotune=False)
    ctx.close()  # the handles keep the context alive
    x = f.solve(b)
    assert np.linalg.norm(x - xt) / np.linalg.norm(xt) <= 1e-9
    bt.run()
    assert (bt.relres() <= RES_TOL).all()
    f.release()
    bt.destroy()


def test_batch_rejects_invalid_system():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    draws = [(1000, 2, 1, 1.5), (1000, 3, 1, 1.5)]
    hb = W.gen_batch(draws, seed=14)
    hb.colind[int(hb.nz_off[1]) + 10] = 5000  # column out of range in system 1
    t, systems = _device_batch(hb, torch, dev)
    with pytest.raises(hs.SpikeError) as e:
        hs.Batch(systems, autotune=False)
    assert e.value.name == "csr" and "system 1" in str(e.value)
