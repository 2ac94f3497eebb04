"""Host-side logic of batches and workloads, checked without a GPU.

* the batch partition rule (spike_batch_partitions): at least one partition
  per system, at least two tiles per partition when the system allows it,
  nearest count to the target length;
* the seeded workload draws: ranges, determinism, and the generated systems'
  consistency (b = A x_true) against the oracle's FP64 residual;
* without a device, creating a batch fails loudly.
"""
import numpy as np
import pytest

import hspike_gb300 as hs
from hspike_gb300 import workloads as W
from tests.conftest import has_gpu


def test_partition_rule():
    for n in (1, 7, 63, 64, 65, 1000, 15_000, 65_536):
        for KB in (2, 4, 8, 16, 32, 64):
            for rpp in (1, 32, 512, 2048, 10_000):
                p = hs.batch_partitions(n, KB, rpp)
                assert p >= 1
                if n >= 2 * KB:
                    assert n // p >= 2 * KB  # every partition holds two tiles
                    # nearest count to the target unless clamped by the two-tile rule
                    if p < n // (2 * KB):
                        assert abs(n / p - rpp) <= abs(n / (p + 1) - rpp) + 1e-9 or p == 1
                else:
                    assert p == 1
    assert hs.batch_partitions(0, 32, 512) == 0


def test_batch_draws_ranges_and_determinism():
    d1 = W.batch_draws(4096, seed=4)
    assert d1 == W.batch_draws(4096, seed=4)
    n = np.array([x[0] for x in d1])
    k = np.array([x[1] for x in d1])
    r = np.array([x[2] for x in d1])
    dom = np.array([x[3] for x in d1])
    assert n.min() >= 1000 and n.max() <= 65536
    assert set(k) == set(W.BATCH_K) and set(r) == set(W.BATCH_NRHS)
    assert dom.min() >= 1.1 and dom.max() <= 2.0
    # log-uniform: the median is near the geometric mean of the range
    assert abs(np.log(np.median(n)) - 0.5 * (np.log(1000) + np.log(65536))) < 0.1
    assert 60e6 < n.sum() < 68e6


def test_generated_batch_is_consistent():
    from oracle import oracle
    draws = W.batch_draws(16, seed=21, n_range=(100, 2000)) + [(20, 32, 1, 1.5)]
    hb = W.gen_batch(draws, seed=21)
    for i in range(len(draws)):
        rp, ci, a, xt, b = hb.system(i)
        assert rp[0] == 0 and rp[-1] == len(ci)
        assert oracle.residual(rp, ci, a, xt, b).max() < 1e-14


def test_request_stream():
    rs = W.request_stream(20_000, 0.1, seed=5)
    assert rs == W.request_stream(20_000, 0.1, seed=5)
    assert 1500 < len(rs) < 2500  # Poisson count around 2000
    t = np.array([q.t_arrival for q in rs])
    assert (np.diff(t) > 0).all() and t[-1] < 0.1
    reuse = [q for q in rs if q.reuse_of >= 0]
    assert 0.2 < len(reuse) / len(rs) < 0.4
    for q in reuse:
        src = rs[q.reuse_of]
        assert src.reuse_of == -1 and (q.n, q.k, q.seed) == (src.n, src.k, src.seed)
    for q in rs:
        assert 500 <= q.n <= 2_000_000 and 1 <= q.k <= 128 and 1 <= q.nrhs <= 32


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_batch_without_device_fails_loudly():
    with pytest.raises(hs.SpikeError) as e:
        hs.Batch([(100, 298, 1, 1, 1, 1, 1, 1)])
    assert e.value.name == "no_device"


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_server_without_device_fails_loudly():
    with pytest.raises(hs.SpikeError) as e:
        hs.Server(slots=2)
    assert e.value.name == "no_device"
