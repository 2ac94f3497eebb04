"""The C-ABI boundary, checked without a GPU.

* libspike_gb300.so loads and exports every function and object that
  include/*.h declares (the reference's five entry points of
  OpenMP/spike_interfaces.h:28-72 plus the spike_gb300.h extensions);
* argument errors return SPIKE_ERROR with a detail code instead of aborting
  (the reference aborts: OpenMP/spike_interfaces.c:53-56);
* without a device the solve fails loudly (no CPU fallback).
"""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import hspike_gb300 as hs
from hspike_gb300.build import lib_path
from tests.conftest import ROOT, has_gpu


def declared_symbols():
    names = set()
    for h in ("spike_interfaces.h", "spike_gb300.h", "spike_datatypes.h", "spike_compat.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = "\n".join(line for line in text.splitlines() if not line.lstrip().startswith("#"))
        # function declarations; "(*name)(...)" members of a struct (callbacks) are not symbols
        names |= set(re.findall(r"\b(\w+)\s*\((?!\s*\*)[^;{]*\)\s*;", text))
        names |= set(re.findall(r"extern\s+const\s+\w+\s+(\w+)\s*;", text))
    return names


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path()], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_library_loads_and_exports_every_declared_symbol():
    hs.load()
    decl = declared_symbols()
    assert {"dspike_core_host", "sspike_core_host", "cspike_core_host", "zspike_core_host",
            "dspike_core_host_blocking", "SPIKE_SUCCESS", "SPIKE_ERROR"} <= decl
    missing = decl - exported_symbols()
    assert not missing, f"declared but not exported: {sorted(missing)}"
    assert set(hs.EXPORTS) <= exported_symbols()


def test_status_objects_have_reference_values():
    L = hs.load()
    assert C.c_int.in_dll(L, "SPIKE_SUCCESS").value == 0
    assert C.c_int.in_dll(L, "SPIKE_ERROR").value == 1


def test_only_api_symbols_exported():
    # the CUDA layer is built with hidden visibility; internal spk_* stay private
    ex = exported_symbols()
    assert not any(s.startswith("spk_") for s in ex)
    assert not any(s.startswith("oracle_") for s in ex)


def test_argument_errors_return_spike_error():
    z = np.zeros(1, np.float64)
    i = np.zeros(2, np.int32)
    assert hs.dspike_core_host(-1, 0, 1, i, i, z, z, z) == hs.SPIKE_ERROR
    assert hs.last_error()[0] == 1
    assert hs.dspike_core_host(1, -5, 1, i, i, z, z, z) == hs.SPIKE_ERROR
    # n == 0 or nrhs == 0 is an empty, successful solve
    assert hs.dspike_core_host(0, 0, 1, i, i, z, z, z) == hs.SPIKE_SUCCESS
    assert hs.dspike_core_host(3, 0, 0, i, i, z, z, z) == hs.SPIKE_SUCCESS
    L = hs.load()
    assert L.dspike_core_host(3, 3, 1, None, None, None, None, None) == hs.SPIKE_ERROR
    assert hs.last_error()[0] == 1


def test_option_validation():
    if not has_gpu():
        pytest.skip("options live on a device context")
    with pytest.raises(hs.SpikeError):
        hs.set_option(hs.SPIKE_OPT_PRECISION, 7)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly():
    rp, ci, a, xt, b = hs.gen_banded(100, 1, 1, 2.0, 1)
    x = np.zeros_like(b, order="F")
    assert hs.dspike_core_host(100, len(ci), 1, ci, rp, a, x, b) == hs.SPIKE_ERROR
    code, msg = hs.last_error()
    assert hs.ERR_NAMES[code] == "no_device", msg
    assert not x.any()  # nothing computed on the host


@pytest.mark.parametrize("lang", ["c99", "c++17"])
def test_public_headers_compile_alone(tmp_path, lang):
    """Every header under include/ compiles on its own and together, warning
    free, as C99 (the reference's dialect) and as C++17."""
    heads = sorted(os.path.basename(h) for h in glob.glob(os.path.join(ROOT, "include", "*.h")))
    for group in [[h] for h in heads] + [heads]:
        ext, cc = (".c", "gcc") if lang == "c99" else (".cpp", "g++")
        src = tmp_path / ("t" + ext)
        src.write_text("".join(f'#include "{h}"\n' for h in group) + "int main(void) { return 0; }\n")
        r = subprocess.run([cc, f"-std={lang}", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                            "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
        assert r.returncode == 0, (group, r.stderr)
