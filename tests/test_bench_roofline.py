"""bench.py's roofline bookkeeping, checked without a GPU.

The compulsory-byte and row-block counts the bench divides by must describe
the workload it times: the CSR it generates, and the row blocks the solver's
plan builds for the caller-set partition rule (floor(n / p) rows each, the
remainder in the last, each padded to whole tiles).
"""
import numpy as np
import pytest

import bench
import hspike_gb300 as hs


def _plan_blocks(n, p, kb):
    """the partition rule stated directly: one entry per partition"""
    size = [n // p] * (p - 1) + [n - (p - 1) * (n // p)]
    return sum((m + kb - 1) // kb for m in size)


@pytest.mark.parametrize("n,p,kb", [(2_000_000, 256, 64), (600_000, 300, 64), (4_000_000, 512, 4),
                                    (100_000, 4, 2), (1_000, 7, 8), (130, 3, 64)])
def test_row_blocks_follow_the_partition_rule(n, p, kb):
    assert bench.row_blocks(n, p, kb) == _plan_blocks(n, p, kb)


def test_row_blocks_of_the_large_band_match_its_band_pass_grid():
    # the band pass of the large band launches one CTA per row block: 31,490
    # (the launch list and the full-size DRAM capture show that grid)
    assert bench.row_blocks(bench.N, bench.P, 64) == 31_490


@pytest.mark.parametrize("n,k", [(1_000, 1), (5_000, 3), (2_000, 64), (300, 64)])
def test_nnz_formula_matches_the_generated_band(n, k):
    rp, ci, a, _, _ = hs.gen_banded(n, k, k, 1.5, 7)
    assert len(ci) == bench.nnz_of(n, k) == int(rp[-1])


def test_compulsory_bytes_read_the_csr_once_and_move_b_and_x():
    n, k, nrhs = 10_000, 8, 3
    nnz = bench.nnz_of(n, k)
    # values (8 B) and column indices (4 B) per entry, the row pointers, b read, x written
    assert bench.alg_bytes(n, k, nrhs) == 12 * nnz + 4 * (n + 1) + 2 * 8 * n * nrhs


def test_traffic_per_block_matches_the_tiles_each_family_must_move():
    """The measured DRAM bytes per 64-row block are within 10 % of the FP32
    tiles (and CSR rows) the kernels must read and write: far below would
    mean the capture missed traffic or the per-block division is wrong, far
    above would mean re-reads."""
    tile = 64 * 64 * 4
    must = {"factor_fwd": 7 * tile,   # LU: D, F, E in, L/U and G/H out; W sweep: L in, spike tile out
            "rhs_sweeps": 3 * tile}   # L / G / E read once per application
    for fam, need in must.items():
        got = bench.TRAFFIC_PER_BLOCK[fam]
        assert 0.9 * need <= got <= 1.1 * need, (fam, got, need)
    # the band pass reads the CSR rows of a block (129 entries of 12 B per row
    # in the large band) and writes four tiles
    band_need = 64 * (129 * 12 + 4) + 4 * tile
    assert 0.9 * band_need <= bench.TRAFFIC_PER_BLOCK["band_tiles"] <= 1.1 * band_need
