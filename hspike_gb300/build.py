"""Build recipe for the native libraries, in-tree under ``hspike_gb300/_build``.

* ``libspike_gb300.so`` -- the product: the C host layer (``spike_host.c``,
  gcc) and the sm_103a kernels (``spike_*.cu``, nvcc, one translation unit
  per kernel family, compiled in parallel), linked with the static CUDA
  runtime.  It exports exactly the symbols of ``include/spike_interfaces.h``
  and ``include/spike_gb300.h`` (plus ``SPIKE_SUCCESS`` / ``SPIKE_ERROR``).
* ``libspike_gen.so`` -- the seeded synthetic-system generator.

Only ``-gencode arch=compute_103a,code=sm_103a`` is emitted: the kernels are
written for GB300 and nothing else.  Portable host flags only (the library is
rebuilt on x86 and on Arm hosts).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["spike_factor.cu", "spike_twist.cu", "spike_apply.cu", "spike_reduced.cu", "spike_util.cu",
              "spike_noalloc.cu"]
C_SOURCES = ["spike_host.c", "spike_batch.c", "spike_serve.c", "spike_reorder.c", "spike_compat.c", "spike_shard.c"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def lib_path() -> str:
    return os.path.join(OUT, "libspike_gb300.so")


def gen_path() -> str:
    return os.path.join(OUT, "libspike_gen.so")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    if verbose and r.stdout.strip():
        print(r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers += [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
    inc = ["-I", CSRC, "-I", INCLUDE]
    nv = nvcc()
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        if _stale(o, [s] + headers):
            cmd = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
                   "-fvisibility=hidden", *inc, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".c", ".o"))
        if _stale(o, [s] + headers):
            jobs.append(["gcc", "-O2", "-std=gnu11", "-fPIC", "-pthread", "-Wall", "-Wextra", "-Wno-unused-parameter",
                         *inc, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(lambda c: _run(c, verbose), jobs))
        if ptxas_info:
            for o in outs:
                print(o)
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s in CU_SOURCES]
    objs += [os.path.join(OUT, s.replace(".c", ".o")) for s in C_SOURCES]
    so = lib_path()
    if _stale(so, objs):
        tmp = so + ".tmp"
        _run([nv, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lm", "-lpthread"], verbose)
        os.replace(tmp, so)
    gsrc = os.path.join(CSRC, "spike_gen.c")
    gso = gen_path()
    if _stale(gso, [gsrc]):
        tmp = gso + ".tmp"
        _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", gsrc, "-o", tmp, "-lm"], verbose)
        os.replace(tmp, gso)
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
