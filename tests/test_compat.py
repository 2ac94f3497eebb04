"""The reference's matrix helpers, CSR files and directSolver_* plugin
(include/spike_compat.h).

Host checks (no device): matrix_LoadCSR reads every real golden fixture
exactly as the Python fixture reader does, with the bandwidth of
matrix_ComputeBandwidth (ku = 2, kl = 4 for Tests/bandwidth/banded.bin,
Tests/bandwidth/readme.txt); matrix_SaveCSR / matrix_ExportBinary round-trip
byte for byte, and so do block files and raw vector files; a complex (planar) file, a truncated file and a missing file are
errors, not misreads; the plugin refuses to start without a device.  GPU
checks: factor once and solve several right-hand-side blocks (the reference's
Configure/Factorize/SolveForRHS sequence, OpenMP/spike_superlu.c:112-272),
refactor a second matrix in the same handler, and the one-shot
directSolver_Solve, each against the oracle's residual and the true solution;
and a C program written like the reference's drivers (tests/c/compat_driver.c)
compiles against include/, links, and solves the reference's fixtures.
"""
import glob
import os
import subprocess

import numpy as np
import pytest

import hspike_gb300 as hs
from hspike_gb300.fixtures import load_csr as py_load_csr
from tests.conftest import GOLDEN, ROOT, has_gpu

REAL = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.bin")))


@pytest.mark.parametrize("path", REAL, ids=[os.path.basename(p) for p in REAL])
def test_load_csr_matches_the_fixture_reader(path):
    from oracle import oracle
    rp, ci, a, ku, kl = hs.load_csr(path)
    A = py_load_csr(path)
    assert np.array_equal(rp, A.rowptr) and np.array_equal(ci, A.colind)
    assert np.array_equal(a.view(np.uint64), A.aij.view(np.uint64))
    assert (ku, kl) == oracle.bandwidth(A.rowptr, A.colind)
    assert (ku, kl) == hs.compute_bandwidth(rp, ci)


def test_bandwidth_of_the_reference_fixture():
    rp, ci, _, ku, kl = hs.load_csr(os.path.join(GOLDEN, "bandwidth__banded.bin"))
    assert (ku, kl) == (2, 4)


def test_bandwidth_of_a_diagonal_and_an_empty_matrix():
    assert hs.compute_bandwidth(np.arange(6, dtype=np.int32), np.arange(5, dtype=np.int32)) == (0, 0)
    assert hs.compute_bandwidth(np.zeros(4, np.int32), np.zeros(0, np.int32)) == (0, 0)


def test_save_csr_round_trip_is_byte_exact(tmp_path):
    src = os.path.join(GOLDEN, "heptadiagonal__medium.bin")
    rp, ci, a, _, _ = hs.load_csr(src)
    out = str(tmp_path / "copy.bin")
    hs.save_csr(out, rp, ci, a)
    assert open(out, "rb").read() == open(src, "rb").read()


def test_save_and_load_a_generated_system(tmp_path):
    rp, ci, a, _, _ = hs.gen_banded(5000, 7, 3, 1.5, 11)
    out = str(tmp_path / "gen.bin")
    hs.save_csr(out, rp, ci, a)
    rp2, ci2, a2, ku, kl = hs.load_csr(out)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2) and np.array_equal(a, a2)
    assert (ku, kl) == (7, 3)


@pytest.mark.parametrize("name", ["spike__penta_15.z", "complex16__penta_15.z"])
def test_complex_file_is_refused_not_misread(name):
    with pytest.raises(hs.SpikeError) as e:
        hs.load_csr(os.path.join(GOLDEN, name))
    assert e.value.name == "argument" and "complex" in str(e.value)


def test_truncated_and_missing_files_are_errors(tmp_path):
    raw = open(os.path.join(GOLDEN, "heptadiagonal__small.bin"), "rb").read()
    cut = tmp_path / "cut.bin"
    cut.write_bytes(raw[:-9])
    with pytest.raises(hs.SpikeError) as e:
        hs.load_csr(str(cut))
    assert e.value.name == "csr"
    with pytest.raises(hs.SpikeError) as e:
        hs.load_csr(str(tmp_path / "absent.bin"))
    assert e.value.name == "argument"


def test_block_file_round_trip(tmp_path):
    a = np.asfortranarray(np.random.default_rng(5).standard_normal((9, 4)))
    out = str(tmp_path / "blk.bin")
    hs.save_block(out, a, ku=2, kl=3, type_=1, section=2)
    raw = open(out, "rb").read()
    assert np.array_equal(np.frombuffer(raw[:24], np.int32), [1, 2, 9, 4, 2, 3])
    assert np.array_equal(np.frombuffer(raw[24:], np.float64), a.ravel(order="F"))
    b, type_, section, ku, kl = hs.load_block(out)
    assert np.array_equal(b, a) and (type_, section, ku, kl) == (1, 2, 2, 3)
    (tmp_path / "short.bin").write_bytes(raw[:-8])
    with pytest.raises(hs.SpikeError) as e:
        hs.load_block(str(tmp_path / "short.bin"))
    assert e.value.name == "csr"
    with pytest.raises(hs.SpikeError):
        hs.load_block(str(tmp_path / "absent.bin"))


def test_raw_vector_files(tmp_path):
    perm = np.random.default_rng(6).permutation(50).astype(np.int32)
    rhs = np.linspace(-1, 1, 50)
    (tmp_path / "p.bin").write_bytes(perm.tobytes())
    (tmp_path / "b.bin").write_bytes(rhs.tobytes())
    assert np.array_equal(hs.load_vector(str(tmp_path / "p.bin"), 50, permutation=True), perm)
    assert np.array_equal(hs.load_vector(str(tmp_path / "b.bin"), 50), rhs)
    with pytest.raises(hs.SpikeError):
        hs.load_vector(str(tmp_path / "b.bin"), 51)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_plugin_without_device_fails_loudly():
    with pytest.raises(hs.SpikeError) as e:
        hs.DirectSolver()
    assert e.value.name == "no_device"
    rp, ci, a, xt, b = hs.gen_banded(200, 2, 2, 2.0, 3)
    with pytest.raises(hs.SpikeError) as e:
        hs.direct_solve(rp, ci, a, b)
    assert e.value.name == "no_device"


def _driver(tmp_path):
    """Compile tests/c/compat_driver.c against include/ and the built library."""
    from hspike_gb300.build import lib_path
    exe = str(tmp_path / "compat_driver")
    lib = lib_path()
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "compat_driver.c"), "-o", exe, lib,
                    "-Wl,-rpath," + os.path.dirname(lib), "-lm"], check=True, capture_output=True, text=True)
    return exe


def test_reference_style_driver_compiles_and_links(tmp_path):
    assert os.access(_driver(tmp_path), os.X_OK)


def _relres(rp, ci, a, x, b):
    from oracle import oracle
    return oracle.residual(rp, ci, a, np.asfortranarray(x.reshape(len(rp) - 1, -1)),
                           np.asfortranarray(b.reshape(len(rp) - 1, -1))).max()


@pytest.mark.gpu
def test_plugin_factor_once_solve_many():
    n, k = 40_000, 8
    rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, 21, nrhs=5)
    with hs.DirectSolver(max_nrhs=2) as ds:
        ds.factorize(rp, ci, a)
        for _ in range(2):
            x = ds.solve(b)  # 5 columns in passes of 2, 2, 1
            assert _relres(rp, ci, a, x, b) <= 1e-12
            assert np.linalg.norm(x - xt) / np.linalg.norm(xt) <= 1e-9
        x1 = ds.solve(b[:, 3])  # refinement stops per pass, so a lone column may take another sweep
        assert np.linalg.norm(x1 - x[:, 3]) / np.linalg.norm(x[:, 3]) <= 1e-10
        st = ds.stats
        assert st.rhs_block_count == 7 and st.rhs_column_count == 11
        assert st.factor_t > 0 and st.solve_t > 0
        # a second matrix in the same handler replaces the first factors
        rp2, ci2, a2, xt2, b2 = hs.gen_banded(3000, 3, 5, 1.5, 22)
        ds.factorize(rp2, ci2, a2)
        x2 = ds.solve(b2)
        assert _relres(rp2, ci2, a2, x2, b2) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["heptadiagonal__medium.bin", "solve_small__tridiagonal.bin",
                                  "bandwidth__banded.bin"])
def test_plugin_on_reference_fixtures(name):
    rp, ci, a, _, _ = hs.load_csr(os.path.join(GOLDEN, name))
    n = len(rp) - 1
    b = np.ones(n)
    x = hs.direct_solve(rp, ci, a, b)
    A = py_load_csr(os.path.join(GOLDEN, name)).to_dense()
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) <= 1e-9
    assert _relres(rp, ci, a, x, b) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name,nrhs,max_nrhs", [("heptadiagonal__medium.bin", 5, 2),
                                                ("solve_small__tridiagonal.bin", 1, 64)])
def test_reference_style_driver_runs(tmp_path, name, nrhs, max_nrhs):
    r = subprocess.run([_driver(tmp_path), os.path.join(GOLDEN, name), str(nrhs), str(max_nrhs)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    ku, kl, rel = r.stdout.split()
    A = py_load_csr(os.path.join(GOLDEN, name))
    from oracle import oracle
    assert (int(ku), int(kl)) == oracle.bandwidth(A.rowptr, A.colind)
    assert float(rel) <= 1e-12
    assert f"{2 * nrhs} columns" in r.stderr  # directSolver_ShowStatistics: two passes of nrhs


@pytest.mark.gpu
def test_plugin_errors_are_reported():
    with hs.DirectSolver() as ds:
        with pytest.raises(hs.SpikeError) as e:
            ds.solve(np.ones(4))  # no factorization yet
        assert e.value.name == "handle"
        with pytest.raises(hs.SpikeError):
            ds.factorize(np.array([0, 1, 5], np.int32), np.array([0, 1], np.int32), np.ones(2))
