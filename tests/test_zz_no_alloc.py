"""The solve that allocates nothing (spike_dsolve_device_noalloc), through the C ABI.

Some callers cannot allocate device memory while they solve: programs whose
own pool allocator has taken the device heap, latency-critical loops that
cannot absorb the device-wide synchronisation of cudaFree, plugin hosts that
do not let a library allocate on their behalf.  They get a solve whose
temporaries all live in one fixed, per-device workspace that the library keeps
for the life of the process.  Each case here calls it twice in a row (two
right-hand sides, so the second call runs on the first call's leftovers in the
shared workspace) and compares it with the allocating entry point
spike_dsolve_device, within the tolerance of the other GPU parity tests.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  It passes alone in a fresh
process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import hspike_gb300 as hs

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-9  # same bar as the other GPU parity tests
RES_TOL = 1e-12


def _lib():
    L = hs.load()
    f = L.spike_dsolve_device_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L


def _relerr(x, ref):
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


# (n, k, nrhs): 8-row tiles; 32- and 64-row tiles (two-sided-capable bands,
# 64 partitions at most) that still fit the workspace; more right-hand sides
# than one internal pass takes (64), so several passes share the workspace.
CASES = [(20_000, 8, 2), (16_000, 24, 2), (4_000, 64, 3), (5_000, 8, 70)]


@pytest.mark.parametrize("n,k,nrhs", CASES)
def test_noalloc_matches_allocating_solve_twice_in_a_row(n, k, nrhs):
    torch = pytest.importorskip("torch")
    from oracle import oracle

    L = _lib()
    dev = torch.device("cuda:0")
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed=4242 + k, nrhs=nrhs)
    t_rp, t_ci, t_a = (torch.from_numpy(v).to(dev) for v in (rp, ci, a))
    stream = torch.cuda.current_stream(dev)

    # reference: the existing allocating device entry point
    ctx = hs.Context()
    ctx.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(7)
    rhs = [b, rng.standard_normal((n, nrhs))]  # two calls in a row, different right-hand sides
    for call, bb in enumerate(rhs):
        t_b = torch.from_numpy(np.ascontiguousarray(bb.T)).to(dev)
        t_ref = torch.zeros_like(t_b)
        ctx.solve_device(n, len(ci), nrhs, t_ci.data_ptr(), t_rp.data_ptr(), t_a.data_ptr(), t_ref.data_ptr(),
                         t_b.data_ptr())
        t_x = torch.full_like(t_b, float("nan"))
        rc = L.spike_dsolve_device_noalloc(n, len(ci), nrhs, t_ci.data_ptr(), t_rp.data_ptr(), t_a.data_ptr(),
                                           t_x.data_ptr(), t_b.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert rc == hs.SPIKE_SUCCESS, hs.last_error()
        torch.cuda.synchronize()
        x = t_x.cpu().numpy().T
        ref = t_ref.cpu().numpy().T
        assert np.isfinite(x).all()
        assert _relerr(x, ref) <= ERR_TOL, (call, _relerr(x, ref))
        assert oracle.residual(rp, ci, a, x, bb).max() <= RES_TOL
        if call == 0:
            assert _relerr(x, xt) <= 1e-10
    ctx.close()


def test_noalloc_rejects_a_system_larger_than_its_workspace():
    torch = pytest.importorskip("torch")
    L = _lib()
    dev = torch.device("cuda:0")
    n, k = 200_000, 32  # needs far more than the fixed workspace
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed=5)
    t_rp, t_ci, t_a = (torch.from_numpy(v).to(dev) for v in (rp, ci, a))
    t_b = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev)
    t_x = torch.zeros_like(t_b)
    rc = L.spike_dsolve_device_noalloc(n, len(ci), 1, t_ci.data_ptr(), t_rp.data_ptr(), t_a.data_ptr(),
                                       t_x.data_ptr(), t_b.data_ptr(), None)
    assert rc == hs.SPIKE_ERROR
    code, msg = hs.last_error()
    assert hs.ERR_NAMES[code] == "memory" and "workspace" in msg, msg
