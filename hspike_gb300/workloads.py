"""Seeded synthetic workloads beyond the single large system.

* ``batch_draws`` -- the batched-uneven workload: ``count`` independent real
  banded systems, n log-uniform in [1,000, 65,536], k = kl = ku drawn from
  {1, 2, 3, 8, 32}, nrhs from {1, 4}, dominance U[1.1, 2.0].
* ``gen_batch`` -- the systems of a draw, generated into a few large host
  arrays (one slice per system) so that they move to the device in a handful
  of copies.
* ``request_stream`` -- the serving workload: Poisson arrivals; per request n
  log-normal (median 20,000, sigma 1, clipped to [500, 2,000,000]), k uniform
  in {1..128}, nrhs uniform in {1..32}, dominance 1.05, and a fraction of
  requests that reuse an earlier request's matrix with a fresh right-hand
  side.

Every draw comes from ``numpy.random.default_rng(seed)`` in a fixed order, and
every matrix from the counter-based generator of ``csrc/spike_gen.c``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _gen

BATCH_K = (1, 2, 3, 8, 32)
BATCH_NRHS = (1, 4)


def nnz_banded(n: int, ku: int, kl: int) -> int:
    """entries of a full band: n rows, ku super- and kl sub-diagonals"""
    ku, kl = min(ku, n - 1), min(kl, n - 1)
    return n * (ku + kl + 1) - ku * (ku + 1) // 2 - kl * (kl + 1) // 2


def batch_draws(count: int, seed: int = 4, n_range=(1_000, 65_536), ks=BATCH_K, nrhs_set=BATCH_NRHS,
                dom_range=(1.1, 2.0)):
    """(n, k, nrhs, dominance) per system, drawn in that order per system."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(n_range[0]), np.log(n_range[1])
    out = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(lo, hi)))
        k = int(rng.choice(ks))
        nrhs = int(rng.choice(nrhs_set))
        dom = float(rng.uniform(*dom_range))
        out.append((n, k, nrhs, dom))
    return out


@dataclass
class HostBatch:
    """A batch in host memory: system i's arrays are slices at the offsets."""
    draws: list
    rowptr: np.ndarray
    colind: np.ndarray
    aij: np.ndarray
    x_true: np.ndarray
    b: np.ndarray
    rp_off: np.ndarray  # (count,) offsets into rowptr (n+1 entries each)
    nz_off: np.ndarray  # (count,) offsets into colind / aij
    v_off: np.ndarray   # (count,) offsets into x_true / b (n * nrhs each)

    def system(self, i):
        n, k, nrhs, dom = self.draws[i]
        nnz = nnz_banded(n, k, k)
        rp = self.rowptr[self.rp_off[i]:self.rp_off[i] + n + 1]
        ci = self.colind[self.nz_off[i]:self.nz_off[i] + nnz]
        a = self.aij[self.nz_off[i]:self.nz_off[i] + nnz]
        xt = self.x_true[self.v_off[i]:self.v_off[i] + n * nrhs].reshape((n, nrhs), order="F")
        b = self.b[self.v_off[i]:self.v_off[i] + n * nrhs].reshape((n, nrhs), order="F")
        return rp, ci, a, xt, b


def _align(v, a=32):
    return (v + a - 1) // a * a


def gen_batch(draws, seed: int = 4, alloc=None) -> HostBatch:
    """Generate every system of ``draws``; system i uses generator seed
    ``seed * 1_000_003 + i``.  Slices start on 256-byte boundaries."""
    alloc = alloc or (lambda shape, dtype: np.empty(shape, dtype))
    count = len(draws)
    rp_off = np.zeros(count, np.int64)
    nz_off = np.zeros(count, np.int64)
    v_off = np.zeros(count, np.int64)
    R = Z = V = 0
    for i, (n, k, nrhs, _) in enumerate(draws):
        rp_off[i], nz_off[i], v_off[i] = R, Z, V
        R = _align(R + n + 1, 64)
        Z = _align(Z + nnz_banded(n, k, k), 64)
        V = _align(V + n * nrhs, 32)
    rowptr = alloc((max(R, 1),), np.int32)
    colind = alloc((max(Z, 1),), np.int32)
    aij = alloc((max(Z, 1),), np.float64)
    x_true = alloc((max(V, 1),), np.float64)
    b = alloc((max(V, 1),), np.float64)
    G = _gen()
    addr = lambda arr, off: C.c_void_p(arr.ctypes.data + int(off) * arr.itemsize)
    for i, (n, k, nrhs, dom) in enumerate(draws):
        nnz = int(G.spike_gen_rowptr(n, k, k, addr(rowptr, rp_off[i])))
        assert nnz == nnz_banded(n, k, k)
        G.spike_gen_fill(n, k, k, float(dom), int(seed * 1_000_003 + i), 0, nrhs, addr(rowptr, rp_off[i]),
                         addr(colind, nz_off[i]), addr(aij, nz_off[i]), addr(x_true, v_off[i]), addr(b, v_off[i]))
    return HostBatch(draws, rowptr, colind, aij, x_true, b, rp_off, nz_off, v_off)


def batch_bytes(draws) -> int:
    """compulsory bytes of one batch solve: every CSR once, b, x"""
    tot = 0
    for n, k, nrhs, _ in draws:
        tot += 12 * nnz_banded(n, k, k) + 4 * (n + 1) + 16 * n * nrhs
    return tot


# ---------------------------------------------------------------- serving
@dataclass
class Request:
    rid: int
    t_arrival: float  # seconds from the start of the stream
    n: int
    k: int
    nrhs: int
    dom: float
    seed: int         # generator seed of the matrix
    reuse_of: int     # -1, or the request whose matrix (and factors) this one reuses
    rhs_seed: int     # seed of the fresh right-hand side


def request_stream(rate: float, duration: float, seed: int = 5, median_n=20_000, sigma=1.0, n_clip=(500, 2_000_000),
                   k_max=128, nrhs_max=32, dom=1.05, reuse=0.3, max_requests=None):
    """Poisson arrivals at ``rate`` per second for ``duration`` seconds."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration or (max_requests is not None and len(out) >= max_requests):
            break
        rid = len(out)
        reuse_of = -1
        if out and rng.uniform() < reuse:
            reuse_of = int(rng.integers(0, len(out)))
            while out[reuse_of].reuse_of >= 0:  # reuse the original matrix
                reuse_of = out[reuse_of].reuse_of
        n = int(np.clip(np.exp(np.log(median_n) + sigma * rng.standard_normal()), *n_clip))
        k = int(rng.integers(1, k_max + 1))
        nrhs = int(rng.integers(1, nrhs_max + 1))
        if reuse_of >= 0:
            src = out[reuse_of]
            n, k = src.n, src.k
        out.append(Request(rid, t, n, k, nrhs, dom, seed * 1_000_003 + (reuse_of if reuse_of >= 0 else rid),
                           reuse_of, seed * 7_000_003 + rid))
    return out
