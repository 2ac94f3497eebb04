"""The host check that decides whether a solve with host arrays may leave the
column indices on the host (spike_csr_full_band, the same row test the solve's
worker threads run range by range).  A false "full band" would make the device
derive wrong columns, so it is compared here, on the CPU, with a plain numpy
statement of the layout on every shape of row the check's 8-wide vector loop
and its scalar tail meet, and on single-entry corruptions of each kind.
"""
import numpy as np
import pytest

import hspike_gb300 as hs


def full_band_np(rp, ci, ku, kl):
    """Row r holds exactly max(0, r - kl) .. min(n - 1, r + ku), in order."""
    n = len(rp) - 1
    if n == 0:
        return len(ci) == 0
    if rp[0] != 0 or rp[-1] != len(ci):
        return False
    r = np.arange(n)
    c0, c1 = np.maximum(0, r - kl), np.minimum(n - 1, r + ku)
    if not np.array_equal(np.diff(rp), c1 - c0 + 1):
        return False
    want = np.concatenate([np.arange(a, b + 1) for a, b in zip(c0, c1)]).astype(np.int32)
    return np.array_equal(ci, want)


@pytest.mark.parametrize("ku,kl", [(0, 0), (1, 1), (2, 4), (3, 3), (4, 3), (7, 0), (0, 9), (12, 5), (16, 16),
                                   (21, 30)])
def test_generated_bands_pass_and_other_bandwidths_fail(ku, kl):
    for n in (1, 2, 5, 37, 300):
        rp, ci, _, _, _ = hs.gen_banded(n, ku, kl, 1.5, 7)
        assert hs.csr_full_band(rp, ci, ku, kl) and full_band_np(rp, ci, ku, kl)
        for du, dl in ((1, 0), (0, 1), (-1, 0), (0, -1)):
            u, l = ku + du, kl + dl
            if u < 0 or l < 0:
                continue
            assert hs.csr_full_band(rp, ci, u, l) == full_band_np(rp, ci, u, l)


def test_single_corruptions_are_caught():
    rng = np.random.default_rng(11)
    checked = 0
    for case in range(400):
        n = int(rng.integers(2, 200))
        ku, kl = int(rng.integers(0, 20)), int(rng.integers(0, 20))
        rp, ci, _, _, _ = hs.gen_banded(n, ku, kl, 1.5, case)
        rp, ci = rp.copy(), ci.copy()
        kind = case % 5
        r = int(rng.integers(0, n))
        t0, t1 = int(rp[r]), int(rp[r + 1])
        if kind == 0:  # one column index off by one
            t = int(rng.integers(t0, t1))
            ci[t] += 1 if rng.random() < 0.5 else -1
        elif kind == 1:  # two entries of a row swapped
            if t1 - t0 < 2:
                continue
            a, b = rng.choice(np.arange(t0, t1), 2, replace=False)
            ci[[a, b]] = ci[[b, a]]
        elif kind == 2:  # an entry moved to the next row (row lengths change, nnz does not)
            if r == n - 1 or t1 - t0 < 2:
                continue
            rp[r + 1] -= 1
        elif kind == 3:  # a row pointer that leaves the arrays
            if r + 1 == n:
                continue
            rp[r + 1] = len(ci) + 3
        else:  # row pointers that do not start at 0
            rp[0] = 1
        assert not full_band_np(rp, ci, ku, kl)
        assert hs.csr_full_band(rp, ci, ku, kl) is False
        checked += 1
    assert checked > 300


def test_empty_and_diagonal_and_bad_arguments():
    assert hs.csr_full_band(np.zeros(1, np.int32), np.zeros(0, np.int32), 0, 0)
    assert hs.csr_full_band(np.arange(4, dtype=np.int32), np.arange(3, dtype=np.int32), 0, 0)
    assert not hs.csr_full_band(np.arange(4, dtype=np.int32), np.array([0, 2, 1], np.int32), 0, 0)
    # bandwidths past the matrix edge mean the edge (no overflow in r + ku)
    rp, ci, _, _, _ = hs.gen_banded(6, 5, 5, 1.5, 3)
    assert hs.csr_full_band(rp, ci, 2**31 - 1, 2**31 - 1)
    assert hs.csr_full_band(rp, ci, 5, 100)
    with pytest.raises(hs.SpikeError) as e:
        hs.csr_full_band(np.arange(4, dtype=np.int32), np.arange(3, dtype=np.int32), -1, 0)
    assert e.value.name == "argument"
