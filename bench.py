"""Benchmark: SPIKE solves/s on the large-band workload (n = 2,000,000,
kl = ku = 64, 256 partitions, 1 right-hand side, float64 CSR, dominance 1.5).

One step = one complete solve of A x = b from CSR already in HBM: analysis,
partition + block LU + spikes, reduced system, right-hand-side sweeps and FP64
iterative refinement until ||b - A x|| / ||b|| <= 1e-12.  ``value`` is that
rate for the mixed-precision path (FP32 factors, FP64 residual / update /
reduced solve); the plain-FP64 rate, nrhs = 16, the end-to-end rate through
the reference's C entry point ``dspike_core_host`` with host buffers, the
per-kernel-family device times, clocks and the CPU baseline (the CPU oracle,
a restatement of the reference path, on a sample of the same workload) ride
along in the same JSON line.

    python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "solves/s & HBM GB/s at resid≤1e-12, mixed vs plain FP64 on 1 GPU; p50/p99 ms"
N, K_BAND, P, NRHS, DOM, SEED = 2_000_000, 64, 256, 1, 1.5, 2
# the CPU arm's caps: one step is a full CPU solve of the workload
REF_MAX_STEPS, REF_MAX_WARMUP = 20, 3
WORKLOAD = (f"large-band real SPIKE: n={N:,} kl=ku={K_BAND} partitions={P} nrhs={NRHS} float64 CSR, "
            f"dominance {DOM}, off-diagonals U[-1,1], seed {SEED}")


# DRAM bytes (read + write) per row block of each kernel family, from one ncu
# capture of this workload at full size (n = 2,000,000, 31,490 row blocks;
# factor_fwd = k_tw_lu 79,741 + k_tw_sweep 30,961); rhs_sweeps from a capture
# of `bench.py --n 600000 --partitions 300` (same 64-row tiles and partition
# length).  Traffic per launch = this x the launch's row blocks.
TRAFFIC_PER_BLOCK = {"factor_fwd": 110_702, "factor_bwd": 111_898, "band_tiles": 162_757, "rhs_sweeps": 48_796}


def row_blocks(n, p, kb):
    """row blocks of kb rows in the plan of n rows on p caller-set partitions:
    floor(n / p) rows each, the remainder in the last, each padded to a
    multiple of kb"""
    nreg = n // p
    return (p - 1) * (-(-nreg // kb)) + (-(-(n - (p - 1) * nreg) // kb))


def nnz_of(n, k):
    return (2 * k + 1) * n - k * (k + 1)


def alg_bytes(n, k, nrhs):
    """compulsory bytes of one solve: read CSR once, read b, write x"""
    nnz = nnz_of(n, k)
    return 12 * nnz + 4 * (n + 1) + 16 * n * nrhs


def alg_flops(n, k, nrhs, applies, residuals):
    """FP32: block LU + spikes 8 k^2 n, sweeps 4 k n per rhs per application;
    FP64: residual 2 nnz per rhs per sweep."""
    f32 = 8.0 * k * k * n + 4.0 * k * n * nrhs * applies
    f64 = 2.0 * nnz_of(n, k) * nrhs * residuals
    return f32, f64


# --------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples over a timed region:
    start() launches the sampler and returns once its first sample is in (the
    tool is live), begin() marks the region's start, stop() summarises the
    samples taken after the mark."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=50, cmd="nvidia-smi"):
        self.index = index
        self.interval_ms = interval_ms
        self.cmd = cmd
        self.rows = []
        self.mark = 0
        self.proc = None

    def start(self, wait_s=3.0):
        # the requested interval first, the tool's customary 200 ms if that one yields nothing
        for interval in dict.fromkeys((self.interval_ms, 200)):
            try:
                self.proc = subprocess.Popen(
                    [self.cmd, "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                     "-lms", str(interval)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
                self.thread = threading.Thread(target=self._read, daemon=True)
                self.thread.start()
            except Exception:
                self.proc = None
                return
            t0 = time.monotonic()
            while not self.rows and self.proc.poll() is None and time.monotonic() - t0 < wait_s:
                time.sleep(0.005)
            if self.rows or self.proc.poll() is None:
                self.interval_ms = interval
                break
            self.thread.join(timeout=2)
        self.begin()

    def begin(self):
        self.mark = len(self.rows)

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        region = self.rows[self.mark:]
        # a region shorter than the interval may hold no sample: the one just before it stands in
        rows = region or self.rows[-1:]
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(region), "interval_ms": self.interval_ms, "reasons": reasons}


# --------------------------------------------------------------------- CPU baseline
def cpu_baseline(system=None, p=P, keep_x=False):
    """Time the CPU oracle -- the restated reference path (oracle/spike_oracle.c:
    banded partial-pivoting LU per partition, reduced system on R's band,
    implicit retrieval), OpenMP over partitions on every host core -- on the
    whole workload (one solve, a few seconds of wall time).  keep_x: the
    oracle's solution rides along under "x" (the GPU results are compared
    with it)."""
    import hspike_gb300 as hs
    from oracle import oracle

    cores = os.cpu_count() or 1
    if system is None:
        rp, ci, a, xt, b = hs.gen_banded(N, K_BAND, K_BAND, DOM, SEED, nrhs=NRHS)
    else:
        rp, ci, a, b = system
    t0 = time.perf_counter()
    x = oracle.spike(rp, ci, a, b, p=p)
    dt = time.perf_counter() - t0
    rel = float(oracle.residual(rp, ci, a, x, b).max())
    out = {"value": 1.0 / dt, "unit": "solves/s", "cores": cores, "kind": "port",
           "sample": (f"one full solve of the workload by oracle/spike_oracle.c (restated reference SPIKE, "
                      f"banded partial-pivoting LU inner solver, {p} partitions) with {cores} OpenMP threads: "
                      f"{dt:.2f} s, relres {rel:.1e}"),
           "seconds": dt}
    if keep_x:
        out["x"] = x
    return out


def measured_peaks():
    """MEASURED_PEAKS.json (the machine's measured copy bandwidth and GEMM rates), or {}."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)) if os.path.exists(path) else {}


def relerr(x, ref):
    x, ref = np.asarray(x), np.asarray(ref)
    return float(np.linalg.norm(x - ref) / max(np.linalg.norm(ref), 1e-300))


def cpu_one_core(n=N, p=P, parts=32):
    """The oracle on one host core: `parts` partitions of the workload's shape
    (n // p rows each, the same band, dominance and seed) solved as one system,
    the time scaled by p / parts to the whole workload (the partitions are
    independent and the reduced system grows linearly with their count)."""
    import hspike_gb300 as hs
    from oracle import oracle

    parts = max(1, min(parts, p))
    rows = (n // p) * parts
    rp, ci, a, xt, b = hs.gen_banded(rows, K_BAND, K_BAND, DOM, SEED, nrhs=NRHS)
    oracle.set_threads(1)
    try:
        t0 = time.perf_counter()
        x = oracle.spike(rp, ci, a, b, p=parts)
        dt = time.perf_counter() - t0
    finally:
        oracle.set_threads(0)
    rel = float(oracle.residual(rp, ci, a, x, b).max())
    est = dt * p / parts
    return {"value": 1.0 / est, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": (f"{parts} of the {p} partitions ({rows:,} rows, same band) solved by oracle/spike_oracle.c "
                       f"on one thread: {dt:.2f} s, relres {rel:.1e}; x {p / parts:g} for the whole workload = "
                       f"{est:.1f} s per solve")}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle.build_oracle import build as build_oracle

    build_oracle()
    import hspike_gb300 as hs
    from hspike_gb300.build import build

    build()
    n, p = args.n, args.partitions
    rp, ci, a, xt, b = hs.gen_banded(n, K_BAND, K_BAND, DOM, SEED, nrhs=NRHS)
    runs = []
    # each step is one full CPU solve (~2 s on 16 cores); the counts are capped
    # so that the whole reference run stays within a few minutes, and the line
    # reports the counts that actually ran
    steps = max(1, min(args.steps, REF_MAX_STEPS))
    warmup = max(0, min(args.warmup, REF_MAX_WARMUP))
    for _ in range(warmup):
        cpu_baseline((rp, ci, a, b), p)
    for _ in range(steps):
        runs.append(cpu_baseline((rp, ci, a, b), p))
    vals = [r["value"] for r in runs]
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "steps_requested": args.steps, "warmup_requested": args.warmup,
            "timed_s": sum(r["seconds"] for r in runs),
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD if (n, p) == (N, P) else WORKLOAD.replace(f"n={N:,}", f"n={n:,}").replace(
                          f"partitions={P}", f"partitions={p}"), "note": "reference C code cannot be built here (MKL / SuperLU_MT "
                       "absent); its path is timed as the CPU restatement in oracle/"},
            "cpu_baseline": {k: runs[-1][k] for k in ("unit", "cores", "kind", "sample")} | {"value": v},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------- peaks
def sgemm_tflops(torch, dev):
    """FP32 CUDA-core peak as measured here: cuBLAS SGEMM 8192^3 with TF32 off,
    best of 5 (the FP32 analogue of the measured bf16 GEMM peak in
    MEASURED_PEAKS.json)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, device=dev)
    b = torch.randn(8192, 8192, device=dev)
    c = torch.empty(8192, 8192, device=dev)
    for _ in range(2):
        torch.matmul(a, b, out=c)
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b, c
    return 2.0 * 8192 ** 3 / (best / 1000.0) / 1e12


# --------------------------------------------------------------------- batched leg
def batched_leg(torch, dev, hs, count, steps, warmup, autotune=True):
    """The batched-uneven workload: `count` independent systems (n log-uniform
    in [1,000, 65,536], k in {1,2,3,8,32}, nrhs in {1,4}, dominance U[1.1,2.0],
    seed 4), solved by one graph launch per step; mixed precision and plain
    FP64, each with its autotuned schedule.  Device-resident inputs; each step
    is spike_batch_run (graph launch + convergence check)."""
    from hspike_gb300 import workloads as W
    from oracle import oracle

    t0 = time.perf_counter()
    draws = W.batch_draws(count, seed=4)
    hb = W.gen_batch(draws, seed=4)
    t = {k: torch.from_numpy(getattr(hb, k)).to(dev) for k in ("rowptr", "colind", "aij", "b")}
    t["x"] = torch.zeros_like(t["b"])
    systems = [(n, W.nnz_banded(n, k, k), nrhs, t["colind"].data_ptr() + 4 * int(hb.nz_off[i]),
                t["rowptr"].data_ptr() + 4 * int(hb.rp_off[i]), t["aij"].data_ptr() + 8 * int(hb.nz_off[i]),
                t["x"].data_ptr() + 8 * int(hb.v_off[i]), t["b"].data_ptr() + 8 * int(hb.v_off[i]))
               for i, (n, k, nrhs, _) in enumerate(draws)]
    gen_s = time.perf_counter() - t0
    B = W.batch_bytes(draws)
    out = {"workload": f"{count} independent real banded systems, n log-uniform [1000, 65536] (sum "
                       f"{sum(d[0] for d in draws):,}), k in {{1,2,3,8,32}}, nrhs in {{1,4}}, dominance U[1.1,2.0], "
                       f"seed 4", "algorithmic_bytes": B, "setup_s": gen_s}
    stream = torch.cuda.current_stream(dev)
    for name, prec in (("mixed", hs.SPIKE_PRECISION_MIXED), ("fp64", hs.SPIKE_PRECISION_FP64)):
        ctx = hs.Context()
        ctx.set_stream(stream.cuda_stream)
        ctx.set_option(hs.SPIKE_OPT_PRECISION, prec)
        c0 = time.perf_counter()
        bt = hs.Batch(systems, ctx, autotune=autotune)
        create_s = time.perf_counter() - c0
        for _ in range(warmup):
            bt.run()
        k = steps if name == "mixed" else max(1, min(steps, 3))
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(k + 1)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for s in range(k):
            bt.run()
            ev[s + 1].record(stream)
        torch.cuda.synchronize()
        per = [ev[s].elapsed_time(ev[s + 1]) for s in range(k)]
        ms = ev[0].elapsed_time(ev[k]) / k
        inf = bt.info()
        rr = bt.relres()
        # error against x_true, and against the oracle (the restated reference
        # path at its own default of 4 partitions), on a sample of systems
        errs, oerrs = [], []
        for i in range(0, count, max(1, count // 64)):
            n, kk, nrhs, _ = draws[i]
            o = int(hb.v_off[i])
            x = t["x"][o:o + n * nrhs].cpu().numpy()
            xt = hb.x_true[o:o + n * nrhs]
            errs.append(relerr(x, xt))
            if name == "mixed":
                rp_i, ci_i, a_i, _, b_i = hb.system(i)
                xo = oracle.spike(rp_i, ci_i, a_i, b_i, p=4)
                oerrs.append(relerr(x.reshape((n, nrhs), order="F"), xo))
        out[name] = {"value": count / (ms / 1000.0), "unit": "systems/s", "ms_per_step": ms,
                     "batches_per_s": 1000.0 / ms, "hbm_gbs": B / (ms / 1000.0) / 1e9,
                     "p50_ms": statistics.median(per), "p99_ms": float(np.percentile(per, 99)),
                     "relres_max": float(rr.max()), "err_vs_xtrue_max_sampled": max(errs),
                     **({"err_vs_oracle_max_sampled": max(oerrs), "oracle_sampled_systems": len(oerrs)}
                        if oerrs else {}),
                     "groups": inf.groups, "graph_kernel_launches": inf.graph_kernel_launches,
                     "graph_sweeps": inf.graph_sweeps, "extra_sweeps": inf.extra_sweeps,
                     "create_s": create_s, "tune_device_ms": inf.tune_ms,
                     "device_gb": inf.device_bytes / 1e9,
                     "schedule": [{k2: g[k2] for k2 in ("block", "nrhs", "systems", "partitions",
                                                         "rows_per_partition", "graph_sweeps")}
                                  for g in bt.groups()]}
        bt.destroy()
        ctx.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    del t
    torch.cuda.empty_cache()
    return out


# --------------------------------------------------------------------- complex leg
def complex_leg(torch, dev, hs, steps, warmup, n=4_000_000, k=3, nrhs=4, p=512, dom=1.2, seed=3):
    """The complex heptadiagonal workload: n = 4,000,000, kl = ku = 3,
    complex128, re/im off-diagonals U[-1,1], diagonal 1.2 x the row's |sum| x
    e^{i theta}, nrhs = 4, 512 partitions; complex64 factors + complex128
    refinement against plain complex128.  Device-resident inputs."""
    from oracle import oracle

    rp, ci, a, xt, b = hs.gen_banded(n, k, k, dom, seed, complex_=True, nrhs=nrhs)
    nnz = len(ci)
    d_rp, d_ci, d_a = (torch.from_numpy(v).to(dev) for v in (rp, ci, a))
    d_b = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev)
    stream = torch.cuda.current_stream(dev)
    B = 20 * nnz + 4 * (n + 1) + 32 * n * nrhs
    hbm_peak = measured_peaks().get("hbm_gbs", 6800.0)
    # the oracle's complex128 solve of the same system, same partitions
    t0 = time.perf_counter()
    xo = oracle.spike(rp, ci, a, b, p=p)
    oracle_s = time.perf_counter() - t0
    out = {"workload": f"complex heptadiagonal: n={n:,} kl=ku={k} complex128, nrhs={nrhs}, {p} partitions, "
                       f"dominance {dom} x |row sum| x e^(i theta), seed {seed}", "algorithmic_bytes": B,
           "hbm_peak_gbs": hbm_peak, "oracle_s": oracle_s}
    for name, prec in (("mixed", hs.SPIKE_PRECISION_MIXED), ("fp64", hs.SPIKE_PRECISION_FP64)):
        ctx = hs.Context()
        ctx.set_stream(stream.cuda_stream)
        ctx.set_option(hs.SPIKE_OPT_PARTITIONS, p)
        ctx.set_option(hs.SPIKE_OPT_PRECISION, prec)
        d_x = torch.zeros_like(d_b)
        go = lambda: ctx.solve_device(n, nnz, nrhs, d_ci.data_ptr(), d_rp.data_ptr(), d_a.data_ptr(), d_x.data_ptr(),
                                      d_b.data_ptr(), complex_=True)
        for _ in range(warmup):
            go()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for s_ in range(steps):
            go()
            ev[s_ + 1].record(stream)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[steps]) / steps
        x = d_x.cpu().numpy().T
        inf = ctx.info()
        out[name] = {"value": 1000.0 / ms, "unit": "solves/s", "ms_per_step": ms, "hbm_gbs": B / (ms / 1000) / 1e9,
                     "hbm_frac": B / (ms / 1000) / 1e9 / hbm_peak, "relres_max": inf.relres_max,
                     "refine_sweeps": inf.refine_sweeps, "block": inf.block,
                     "err_vs_xtrue": relerr(x, xt), "err_vs_oracle": relerr(x, xo)}
        ctx.close()
        del d_x
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


# --------------------------------------------------------------------- serving leg
def serving_leg(hs, window_s, rate=20_000.0, slots=16, k_max=128, pool=48, sub_frac=0.5, sub_window_s=5.0):
    """The serving stream: Poisson arrivals, per request n log-normal (median
    20,000, sigma 1, clipped to [500, 2,000,000]), k uniform in {1..k_max},
    nrhs uniform in {1..32}, dominance 1.05, 30 % of the requests reusing a
    resident factorization with a fresh right-hand side (seed 5).  A client
    thread submits each request at its arrival time to a server of `slots`
    slots admitting by device footprint.  Two runs:

      saturated   the stated offered rate (20,000/s) for `window_s` seconds of
                  the stream, with a bounded admission queue (2 x slots
                  waiting): what the server cannot take is turned away at once
                  (SPIKE_ERR_BUSY), so latency is service plus a short queue;
      sub-saturation  `sub_frac` of the throughput the saturated run reached,
                  for `sub_window_s` seconds, unbounded queue: p50/p99 are
                  service latency.

    The matrices come from a pool of `pool` systems drawn from the same
    distribution (a request takes entry i mod pool; its nrhs is its own draw;
    a reusing request solves with the entry's resident factorization); the
    pool's n is capped at 500,000 rows to bound host memory (0.07 % of draws
    lie above).  Latency = completion - arrival."""
    from hspike_gb300 import workloads as W
    from oracle import oracle

    t0 = time.perf_counter()
    shapes = W.request_stream(rate, 1e9, seed=5, k_max=k_max, max_requests=pool)
    mats = []
    for q in shapes:
        n = min(q.n, 500_000)
        rp, ci, a, xt, b = hs.gen_banded(n, q.k, q.k, q.dom, q.seed, nrhs=32)
        mats.append((rp, ci, a, b, q.k))
    gen_s = time.perf_counter() - t0

    def run(rate_, duration, max_queue, seed):
        reqs = W.request_stream(rate_, duration, seed=seed, k_max=k_max)
        srv = hs.Server(slots=slots, max_queue=max_queue)
        kept = []
        start = srv.clock()
        for i, q in enumerate(reqs):
            j = i % pool
            rp, ci, a, bb, k = mats[j]
            nr = min(q.nrhs, 32)
            x = np.empty((len(rp) - 1, nr), order="F")
            ta = start + q.t_arrival
            while srv.clock() < ta:
                pass
            t, x = srv.submit(rp, ci, a, bb[:, :nr], x=x, factor_key=j if q.reuse_of >= 0 else -1, bandwidth=k,
                              arrival=ta)
            if not srv.poll(t).done:  # turned-away requests are done at once; their x is dropped
                kept.append((t, x, j, nr))
        sent = srv.clock() - start
        srv.drain()
        st = srv.stats()
        worst = 0.0
        for t, x, j, nr in kept[::max(1, len(kept) // 12)]:
            s_ = srv.poll(t)
            if s_.done and s_.error_code == 0:
                rp, ci, a, bb, k = mats[j]
                worst = max(worst, float(oracle.residual(rp, ci, a, x, bb[:, :nr]).max()))
        srv.close()
        return {"offered_per_s": rate_, "window_s": duration, "arrivals": len(reqs),
                "submitted_per_s": len(reqs) / sent if sent > 0 else None, "max_queue": max_queue,
                "completed": st.completed, "rejected_busy": st.rejected_busy, "failed": st.failed,
                "rejected_share": st.rejected_busy / max(1, len(reqs)), "value": st.throughput, "unit": "solves/s",
                "p50_ms": st.latency_p50 * 1000, "p99_ms": st.latency_p99 * 1000, "max_ms": st.latency_max * 1000,
                "mean_queue_wait_ms": st.mean_queue_wait * 1000, "factor_hits": st.factor_hits,
                "peak_running": st.peak_running, "relres_max": st.relres_max, "relres_oracle_sampled": worst}

    sat = run(rate, window_s, 2 * slots, 5)
    sub_rate = max(1.0, sub_frac * (sat["value"] or 1.0))
    sub = run(sub_rate, sub_window_s, 0, 6)
    return {"workload": f"Poisson stream: n log-normal median 20000 sigma 1 clipped [500, 2e6] (pool of {pool} systems, "
                        f"n capped at 500,000), k U{{1..{k_max}}}, nrhs U{{1..32}}, dominance 1.05, 30% reuse of a "
                        f"resident factorization, seed 5; {slots} slots",
            "slots": slots, "setup_s": gen_s, "saturated": sat, "sub_saturation": sub,
            "value": sat["value"], "unit": "solves/s", "p50_ms": sub["p50_ms"], "p99_ms": sub["p99_ms"]}


# --------------------------------------------------------------------- sharded arm
def shard_arm(args, torch, hs, world, rank, local):
    """One solve of the workload split over the ranks by partition ranges
    (spike_shard_dsolve: each rank factors its partitions on its GPU, the
    reduced system's tips go to rank 0 and its solution comes back, x halos
    travel between neighbours), host arrays in and out, exchanges over a gloo
    group.  Strong scaling: the same system whatever the rank count; the
    time is the slowest rank's wall clock around each collective solve."""
    import socket

    import torch.distributed as dist

    from hspike_gb300 import shard

    if world == 1 and "MASTER_ADDR" not in os.environ:
        with socket.socket() as s:
            s.bind(("127.0.0.1", 0))
            os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(s.getsockname()[1]), RANK="0", WORLD_SIZE="1")
    torch.cuda.set_device(local % torch.cuda.device_count())
    dist.init_process_group("gloo")
    comm = shard.TorchComm()
    n, p = args.n, args.partitions
    rp, ci, a, xt, b = hs.gen_banded(n, K_BAND, K_BAND, DOM, SEED, nrhs=NRHS)
    part0, part1, row0, row1 = shard.shard_range(n, p, world, rank)
    tdt = {np.int32: torch.int32, np.float64: torch.float64}

    def pinned_copy(arr):
        """the rank's slice in pinned host memory (what a caller that streams
        matrices to the GPU holds), column order kept"""
        out = torch.empty(arr.size, dtype=tdt[arr.dtype.type], pin_memory=True).numpy()
        out[:] = arr.reshape(-1, order="F")
        return out.reshape(arr.shape, order="F")

    lrp, lci, la = (pinned_copy(v) for v in shard.rows_of(rp, ci, a, row0, row1))
    lb = pinned_copy(np.asfortranarray(b[row0:row1]))
    del rp, ci, a
    ctx = hs.Context()
    ctx.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_MIXED)
    for _ in range(args.warmup):
        shard.shard_solve(comm, n, p, lrp, lci, la, lb, ctx=ctx)
    per = []
    for _ in range(args.steps):
        dist.barrier()
        t0 = time.perf_counter()
        x = shard.shard_solve(comm, n, p, lrp, lci, la, lb, ctx=ctx)
        t = torch.tensor([time.perf_counter() - t0], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        per.append(float(t.item()) * 1000.0)
    info = ctx.info()
    sq = torch.tensor([float(np.sum((x - xt[row0:row1]) ** 2)), float(np.sum(xt[row0:row1] ** 2))],
                      dtype=torch.float64)
    dist.all_reduce(sq)
    ms = sum(per) / len(per)
    if rank == 0:
        line = {"metric": METRIC, "value": 1000.0 / ms, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f32 factors / f64 residual+update+reduced",
                "data": "synthetic (seeded generator)",
                "config": {"workload": WORKLOAD.replace(f"n={N:,}", f"n={n:,}").replace(f"partitions={P}",
                                                                                      f"partitions={p}"),
                           "parallelism": f"partition-range shards x{world} (tips gathered to rank 0)",
                           "l2": "inputs larger than the 129 MB L2; no flush"},
                "p50_ms": statistics.median(per), "relres_max": info.relres_max, "refine_sweeps": info.refine_sweeps,
                "err_vs_xtrue": float(np.sqrt(sq[0].item() / sq[1].item())),
                "e2e": {"value": 1000.0 / ms, "unit": "solves/s", "api": "spike_shard_dsolve (host arrays)",
                        "h2d_bytes_per_step": int(lrp.nbytes + lci.nbytes + la.nbytes + lb.nbytes) * world,
                        "d2h_bytes_per_step": int(x.nbytes) * world}}
        print(json.dumps(line), flush=True)
    ctx.close()
    dist.destroy_process_group()
    return 0


# --------------------------------------------------------------------- GPU arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline leg")
    ap.add_argument("--skip-extras", action="store_true", help="mixed-precision device timing only")
    ap.add_argument("--skip-e2e", action="store_true", help="omit the host-buffer end-to-end leg")
    ap.add_argument("--n", "--rows", dest="n", type=int, default=N,
                    help="rows (smaller cases for profiler captures; --rows under torch.distributed.run)")
    ap.add_argument("--partitions", type=int, default=P)
    ap.add_argument("--k", type=int, default=K_BAND,
                    help="half-bandwidth kl = ku (profiler captures of other tile sizes; the roofline figures assume 64)")
    ap.add_argument("--batch", type=int, default=4096, help="systems in the batched leg (0 = skip it)")
    ap.add_argument("--batch-only", action="store_true", help="run only the batched leg (profiler captures)")
    ap.add_argument("--no-autotune", action="store_true", help="batched leg: schedules by rule")
    ap.add_argument("--serve", type=float, default=3.0,
                    help="seconds of the saturated serving stream (0 = skip the serving leg)")
    ap.add_argument("--serve-only", action="store_true", help="run only the serving leg")
    ap.add_argument("--complex-only", action="store_true", help="run only the complex leg")
    ap.add_argument("--skip-complex", action="store_true", help="omit the complex leg")
    ap.add_argument("--shard", action="store_true",
                    help="under torch.distributed.run: one solve of the workload sharded across the ranks "
                         "(spike_shard_dsolve, strong scaling) instead of independent replicas")
    args = ap.parse_args()
    if args.k != K_BAND:
        globals()["K_BAND"] = args.k
    if args.impl == "reference":
        return reference_arm(args)

    import torch

    import hspike_gb300 as hs
    from hspike_gb300.build import build

    build()
    n, p = args.n, args.partitions
    if args.complex_only:
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        torch.cuda.set_device(dev)
        print(json.dumps({"complex": complex_leg(torch, dev, hs, max(1, args.steps), args.warmup)}), flush=True)
        return 0
    if args.serve_only:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"serving": serving_leg(hs, args.serve)}), flush=True)
        return 0
    if args.batch_only:
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        torch.cuda.set_device(dev)
        res = batched_leg(torch, dev, hs, args.batch, max(1, args.steps), args.warmup, not args.no_autotune)
        print(json.dumps({"batched": res}), flush=True)
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.shard:
        return shard_arm(args, torch, hs, world, rank, local)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:  # independent replicas, one per GPU; no data exchange
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- inputs: pinned host buffers (for e2e) and device copies (for value)
    tdt = {np.int32: torch.int32, np.float64: torch.float64, np.complex128: torch.complex128}

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=tdt[np.dtype(dtype).type], pin_memory=True).numpy()

    rp, ci, a, xt, b = hs.gen_banded(n, K_BAND, K_BAND, DOM, SEED + rank, nrhs=NRHS, alloc=pinned)
    nnz = len(ci)
    d_rp, d_ci, d_a = (torch.from_numpy(v).to(dev) for v in (rp, ci, a))
    d_b = torch.from_numpy(b.T.copy()).to(dev).contiguous()  # n x nrhs column-major == nrhs x n row-major
    d_x = torch.zeros_like(d_b)
    stream = torch.cuda.current_stream(dev)
    ctx = hs.Context()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_option(hs.SPIKE_OPT_PARTITIONS, p)
    ctx.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_MIXED)

    def solve(ctx_, d_x_, d_b_, nrhs):
        ctx_.solve_device(n, nnz, nrhs, d_ci.data_ptr(), d_rp.data_ptr(), d_a.data_ptr(), d_x_.data_ptr(),
                          d_b_.data_ptr())

    def timed(ctx_, steps, d_x_, d_b_, nrhs, warmup, clocks=None):
        for _ in range(warmup):
            solve(ctx_, d_x_, d_b_, nrhs)
        barrier()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        launches = 0
        if clocks:
            clocks.start()
        barrier()
        if clocks:
            clocks.begin()
        ev[0].record(stream)
        for s in range(steps):
            solve(ctx_, d_x_, d_b_, nrhs)
            ev[s + 1].record(stream)
            launches += ctx_.info().kernel_launches
        barrier()
        clk = clocks.stop() if clocks else None
        per = [ev[s].elapsed_time(ev[s + 1]) for s in range(steps)]
        total = ev[0].elapsed_time(ev[steps])
        if dist:
            t = torch.tensor([total], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            total = float(t.item())
        return total, per, launches, clk

    # ---- headline: mixed precision, device-resident inputs
    clocks = ClockSampler(local)
    total, per, launches, clk = timed(ctx, args.steps, d_x, d_b, NRHS, args.warmup, clocks)
    info = ctx.info()
    x = d_x.cpu().numpy().T
    err = float(np.linalg.norm(x - xt) / np.linalg.norm(xt))
    ms = total / args.steps
    value = world * args.steps / (total / 1000.0)
    sweeps = info.refine_sweeps
    out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 factors / f64 residual+update+reduced", "data": "synthetic (seeded generator)",
           "config": {"workload": WORKLOAD if (n, p) == (N, P) else WORKLOAD.replace(f"n={N:,}", f"n={n:,}").replace(
                          f"partitions={P}", f"partitions={p}"), "l2": "inputs (3.1 GB CSR) larger than the 129 MB L2; no flush",
                      "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
           "hbm_gbs": alg_bytes(n, K_BAND, NRHS) / (ms / 1000.0) / 1e9,
           "p50_ms": statistics.median(per), "p99_ms": float(np.percentile(per, 99)),
           "relres_max": info.relres_max, "refine_sweeps": sweeps, "err_vs_xtrue": err,
           "gpu_launches": launches, "clocks": clk}
    if rank != 0 and world > 1:
        dist.barrier()
        return 0

    # the CPU oracle's solve of the same system with the same partitions: the
    # CPU baseline's timing, and the reference every GPU result is held to
    xo = cpu = None
    if not args.skip_cpu and world == 1:
        cpu = cpu_baseline((rp, ci, a, b), p, keep_x=True)
        xo = cpu.pop("x")
        out["err_vs_oracle"] = relerr(x, xo)

    if args.serve > 0 and not args.skip_extras:
        # first of the extra legs: its latencies depend on host threads and
        # device memory that the heavier legs below would leave in use
        torch.cuda.empty_cache()
        out["serving"] = serving_leg(hs, args.serve)

    if not args.skip_extras:
        # ---- per-kernel-family device time (CUDA events on the launching stream)
        ctx.set_option(hs.SPIKE_OPT_PHASE_TIMING, 1)
        ctx.phase_times(reset=True)
        for _ in range(3):
            solve(ctx, d_x, d_b, NRHS)
        torch.cuda.synchronize()
        ph = ctx.phase_times(reset=True)
        ctx.set_option(hs.SPIKE_OPT_PHASE_TIMING, 0)
        fams = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1], "share": 0.0} for k, v in ph.items() if v[1]}
        tot = sum(v[0] for v in ph.values())
        for k in fams:
            fams[k]["share"] = ph[k][0] / tot
        dom = max(fams, key=lambda k: ph[k][0])
        peaks = measured_peaks()
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        p32 = sgemm_tflops(torch, dev)
        KB = info.block
        blocks = row_blocks(n, p, KB)
        k = K_BAND
        csr_bytes = 12 * nnz + 4 * (n + 1)
        # per family: (bound, algorithmic work per launch, executed work per launch, units)
        #   factor_fwd: block LU (2 k^2 n) + the W spike's forward sweep (2 k^2 n); it executes
        #               8 KB^3 per row block (two tile products, the tile inverse, the sweep)
        #   factor_bwd: the rest of the spikes (4 k^2 n); executes 8 KB^3 per row block
        #   band_tiles: reads the CSR once, writes three factor-precision tiles per block
        #   residual:   reads the CSR, x and b, writes r (FP64)
        #   rhs_sweeps: reads the L / G / E tiles once per application
        work = {"factor_fwd": ("fp32", 4.0 * k * k * n, 8.0 * KB ** 3 * blocks),
                "factor_bwd": ("fp32", 4.0 * k * k * n, 8.0 * KB ** 3 * blocks),
                "band_tiles": ("hbm", csr_bytes, csr_bytes + 4 * 4 * KB * KB * blocks),
                "residual": ("hbm", csr_bytes + 24 * n * NRHS, csr_bytes + 24 * n * NRHS),
                "rhs_sweeps": ("hbm", 3 * 4 * KB * KB * blocks, 3 * 4 * KB * KB * blocks)}
        dur = fams[dom]["ms_per_launch"] / 1000.0
        bound, alg, exe = work.get(dom, ("hbm", csr_bytes, csr_bytes))
        traffic = TRAFFIC_PER_BLOCK.get(dom)
        if bound == "fp32":
            out["roofline"] = {"bound": "fp32", "kernel": dom, "achieved": alg / dur / 1e12, "peak": p32,
                               "unit": "TFLOP/s", "frac": alg / dur / 1e12 / p32,
                               "traffic": traffic * blocks if traffic else None,
                               "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run (FP32 CUDA "
                                              "cores: the factors are FP32 by design, no tensor-core path)",
                               "algorithmic_tflop_per_launch": alg / 1e12, "executed_tflop_per_launch": exe / 1e12,
                               "executed_frac": exe / dur / 1e12 / p32, "ms_per_launch": dur * 1000.0,
                               "traffic_source": "ncu dram__bytes_read+write per row block of this kernel "
                                                 "(n=2,000,000 capture) x row blocks"}
        else:
            out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": alg / dur / 1e9, "peak": hbm_peak,
                               "unit": "GB/s", "frac": alg / dur / 1e9 / hbm_peak,
                               "traffic": traffic * blocks if traffic else None,
                               "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback",
                               "ms_per_launch": dur * 1000.0}
        for fam, (bd, al, ex) in work.items():
            if fam in fams:
                d = fams[fam]["ms_per_launch"] / 1000.0
                fams[fam]["bound"] = bd
                if bd == "fp32":
                    fams[fam]["alg_tflops"] = al / d / 1e12
                    fams[fam]["frac_of_sgemm"] = al / d / 1e12 / p32
                    fams[fam]["executed_tflops"] = ex / d / 1e12
                else:
                    fams[fam]["alg_gbs"] = al / d / 1e9
                    fams[fam]["frac_of_hbm"] = al / d / 1e9 / hbm_peak
        out["kernel_families"] = fams
        f32, f64 = alg_flops(n, K_BAND, NRHS, 1 + sweeps, 1 + sweeps)
        t_roof = max(alg_bytes(n, K_BAND, NRHS) / (hbm_peak * 1e9), f32 / (p32 * 1e12) + f64 / 1.25e12)
        out["solve_roofline"] = {"t_roof_ms": t_roof * 1000, "frac": t_roof / (ms / 1000.0),
                                 "hbm_frac": alg_bytes(n, K_BAND, NRHS) / (hbm_peak * 1e9) / (ms / 1000.0),
                                 "rule": "max(B_alg/BW_hbm, F32/P32 + F64/P64); BW measured (MEASURED_PEAKS.json), "
                                         "P32 measured SGEMM, P64 1.25 TFLOP/s nominal GB300 FP64",
                                 "p32_tflops": p32, "f32_gflop": f32 / 1e9, "f64_gflop": f64 / 1e9}

        # ---- plain FP64 SPIKE (the denominator of the mixed/plain ratio)
        ctx64 = hs.Context()
        ctx64.set_stream(stream.cuda_stream)
        ctx64.set_option(hs.SPIKE_OPT_PARTITIONS, p)
        ctx64.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_FP64)
        d_x64 = torch.zeros_like(d_b)
        t64, per64, _, _ = timed(ctx64, 3, d_x64, d_b, NRHS, 1)
        i64 = ctx64.info()
        x64 = d_x64.cpu().numpy().T
        out["fp64"] = {"value": 3 / (t64 / 1000.0), "unit": "solves/s", "ms_per_step": t64 / 3,
                       "relres_max": i64.relres_max, "mixed_over_fp64": value / (3 / (t64 / 1000.0)),
                       "err_vs_xtrue": relerr(x64, xt)}
        if xo is not None:
            out["fp64"]["err_vs_oracle"] = relerr(x64, xo)
        ctx64.close()
        del d_x64

        # ---- the reduced system's cyclic reduction in FP64 (SPIKE_OPT_REDUCED_FP64),
        # FP32 partition factors as in the headline: the reference solves R in FP64
        ctxr = hs.Context()
        ctxr.set_stream(stream.cuda_stream)
        ctxr.set_option(hs.SPIKE_OPT_PARTITIONS, p)
        ctxr.set_option(hs.SPIKE_OPT_REDUCED_FP64, 1)
        d_xr = torch.zeros_like(d_b)
        tr, _, _, _ = timed(ctxr, 5, d_xr, d_b, NRHS, 2)
        ir = ctxr.info()
        xr = d_xr.cpu().numpy().T
        ctxr.set_option(hs.SPIKE_OPT_PHASE_TIMING, 1)
        ctxr.phase_times(reset=True)
        for _ in range(3):
            solve(ctxr, d_xr, d_b, NRHS)
        torch.cuda.synchronize()
        phr = ctxr.phase_times(reset=True)
        out["reduced_fp64"] = {"value": 5 / (tr / 1000.0), "unit": "solves/s", "ms_per_step": tr / 5,
                               "relres_max": ir.relres_max, "refine_sweeps": ir.refine_sweeps,
                               "reduced_fp64": ir.reduced_fp64, "err_vs_xtrue": relerr(xr, xt),
                               "reduced_factor_ms": phr["reduced_factor"][0] / max(1, phr["reduced_factor"][1]),
                               "reduced_solve_ms": phr["reduced_solve"][0] / max(1, phr["reduced_solve"][1]),
                               "reduced_factor_ms_fp32": fams.get("reduced_factor", {}).get("ms_per_launch"),
                               "reduced_solve_ms_fp32": fams.get("reduced_solve", {}).get("ms_per_launch")}
        if xo is not None:
            out["reduced_fp64"]["err_vs_oracle"] = relerr(xr, xo)
        ctxr.close()
        del d_xr

        # ---- nrhs = 16
        gen16 = hs.gen_banded(n, K_BAND, K_BAND, DOM, SEED, nrhs=16)
        d_b16 = torch.from_numpy(gen16[4].T.copy()).to(dev)
        d_x16 = torch.zeros_like(d_b16)
        # same matrix (same seed), 16 right-hand sides
        t16, per16, _, _ = timed(ctx, 3, d_x16, d_b16, 16, 1)
        x16 = d_x16.cpu().numpy().T
        out["nrhs16"] = {"value": 3 / (t16 / 1000.0), "unit": "solves/s", "ms_per_step": t16 / 3,
                         "hbm_gbs": alg_bytes(n, K_BAND, 16) / (t16 / 3000.0) / 1e9,
                         "relres_max": ctx.info().relres_max, "err_vs_xtrue": relerr(x16, gen16[3])}
        if not args.skip_cpu:
            from oracle import oracle

            out["nrhs16"]["err_vs_oracle"] = relerr(x16, oracle.spike(rp, ci, a, gen16[4], p=p))
        del d_b16, d_x16, gen16

    if args.batch > 0 and not args.skip_extras:
        out["batched"] = batched_leg(torch, dev, hs, args.batch, max(3, min(args.steps, 10)), 3,
                                     not args.no_autotune)

    if not args.skip_complex and not args.skip_extras:
        out["complex"] = complex_leg(torch, dev, hs, max(3, min(args.steps, 10)), 3)

    # ---- end to end through the reference's C entry point, host buffers
    if not args.skip_e2e:
        hs.set_option(hs.SPIKE_OPT_PARTITIONS, p)
        hs.set_option(hs.SPIKE_OPT_PRECISION, hs.SPIKE_PRECISION_MIXED)
        xh = pinned((n * NRHS,), np.float64).reshape((n, NRHS), order="F")
        e2e_steps = max(1, min(args.steps, 5))
        for _ in range(max(1, args.warmup)):
            hs.dspike_core_host(n, nnz, NRHS, ci, rp, a, xh, b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            rc = hs.dspike_core_host(n, nnz, NRHS, ci, rp, a, xh, b)
            if rc != hs.SPIKE_SUCCESS:
                raise RuntimeError(hs.last_error())
        te = time.perf_counter() - t0
        # with the full band verified on host threads the column indices stay on
        # the host: count the bytes that actually crossed the host link
        implied = hs.get_info().columns_implied == 1
        out["e2e"] = {"value": e2e_steps / te, "unit": "solves/s", "ms_per_step": te * 1000 / e2e_steps,
                      "h2d_bytes_per_step": int(rp.nbytes + (0 if implied else ci.nbytes) + a.nbytes + b.nbytes),
                      "d2h_bytes_per_step": int(xh.nbytes), "api": "dspike_core_host (pinned host buffers)",
                      "columns_implied": implied,
                      "host_threads": int(hs.get_option(hs.SPIKE_OPT_HOST_THREADS)),
                      "err_vs_xtrue": relerr(xh, xt)}
        if xo is not None:
            out["e2e"]["err_vs_oracle"] = relerr(xh, xo)

    if cpu is not None:
        out["cpu_baseline"] = cpu
        try:  # a supplementary figure: its failure must not cost the line
            out["cpu_baseline"]["one_core"] = cpu_one_core(n, p)
        except Exception as e:  # noqa: BLE001
            out["cpu_baseline"]["one_core"] = {"error": f"{type(e).__name__}: {e}"}

    ctx.close()
    if dist:
        dist.barrier()
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
