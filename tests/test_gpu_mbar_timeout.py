"""A bulk-copy wait that runs out ends in a status, not a hang.

The chain kernels stage their tiles by bulk copies and wait on mbarriers with
a bounded number of polls (mbar_wait, spike_common.cuh); a wait that runs
out sets SPK_DEV_ERR_TIMEOUT and the kernel returns, which the host reports as
an error.  Here a kernel waits on a barrier that nothing arrives on: the wait
must give up (in a bounded time) and the context must stay usable -- the next
kernel, whose copy does land, completes its wait.
"""
import ctypes as C
import os
import subprocess

import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def test_wait_on_a_copy_that_never_lands_gives_up(tmp_path):
    from hspike_gb300.build import ARCH, nvcc

    so = str(tmp_path / "libmbar_check.so")
    subprocess.run([nvcc(), *ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                    "-I", os.path.join(ROOT, "hspike_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "mbar_timeout.cu"), "-o", so],
                   check=True, capture_output=True, text=True)
    L = C.CDLL(so)
    L.mbar_check.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_float)]
    L.mbar_check.restype = C.c_int
    flags = (C.c_int * 3)()
    ms = C.c_float()
    assert L.mbar_check(flags, C.byref(ms)) == 0  # no CUDA error: the context survived
    assert flags[0] == 1 and flags[1] == 0  # the wait gave up, and said so
    assert flags[2] == 1  # a later copy's wait succeeds
    assert ms.value < 30_000, ms.value  # bounded
    print(f"wait gave up after {ms.value:.1f} ms")
