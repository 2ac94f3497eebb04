"""Build recipe for the CPU oracle (``oracle/_build/liboracle.so``).

``spike_oracle.c`` is compiled twice into one shared library: once as real
double (``d`` prefix) and once with ``-DORACLE_COMPLEX`` (``z`` prefix).
Portable flags only (the library is rebuilt on x86 and on Arm hosts); -O3
because the reference's arithmetic runs in optimised libraries (MKL,
SuperLU_MT), and ISO C mode keeps floating-point contraction off, so the
results are the same bits as at -O2.

The reference's own C sources cannot be built here (MKL and SuperLU_MT
headers are absent), so there is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build(verbose: bool = False) -> str:
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "spike_oracle.c")
    so = os.path.join(out_dir, "liboracle.so")
    if os.path.exists(so) and os.path.getmtime(so) > os.path.getmtime(src):
        return so
    cflags = ["-O3", "-std=c11", "-fPIC", "-fopenmp", "-Wall", "-Wno-unknown-pragmas"]
    objs = []
    for tag, extra in (("d", []), ("z", ["-DORACLE_COMPLEX"])):
        obj = os.path.join(out_dir, f"spike_oracle_{tag}.o")
        cmd = ["gcc", *cflags, *extra, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        objs.append(obj)
    tmp = so + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-fopenmp", *objs, "-o", tmp, "-lm"])
    os.replace(tmp, so)
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
