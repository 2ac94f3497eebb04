"""The request loop (spike_server_*): continuous batching, admission by device
footprint, resident factors.

The bar: every request's result is the same alone and in the mix -- solved
one at a time on a one-slot server, or concurrently with others on a
four-slot server (requests admitted while others run) -- within
||x_mix - x_alone|| / ||x_alone|| <= 1e-9, and every result meets relres
<= 1e-12 against the oracle's FP64 residual.  Repeat right-hand sides solve
with the resident factorization.
"""
import numpy as np
import pytest

import hspike_gb300 as hs

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-9
RES_TOL = 1e-12


def _requests(count=24, seed=31):
    rng = np.random.default_rng(seed)
    mats = []
    reqs = []
    for i in range(count):
        if mats and rng.uniform() < 0.3:  # a fresh right-hand side for an earlier matrix
            j = int(rng.integers(0, len(mats)))
            rp, ci, a, key = mats[j]
            n = len(rp) - 1
            b = rng.standard_normal((n, int(rng.integers(1, 5))))
            reqs.append((rp, ci, a, b, key))
            continue
        n = int(rng.integers(2_000, 40_000))
        k = int(rng.integers(1, 129))  # 128-row tiles above 64
        nrhs = int(rng.integers(1, 9))
        rp, ci, a, xt, b = hs.gen_banded(n, k, k, 1.5, seed=1000 + i, nrhs=nrhs)
        key = 1000 + i if rng.uniform() < 0.5 else -1
        if key >= 0:
            mats.append((rp, ci, a, key))
        reqs.append((rp, ci, a, b, key))
    return reqs


def _check(req, x):
    from oracle import oracle
    rp, ci, a, b, key = req
    res = oracle.residual(rp, ci, a, x, b).max()
    assert np.isfinite(x).all() and res <= RES_TOL, res


def test_each_result_is_the_same_alone_and_in_the_mix():
    reqs = _requests()
    alone = []
    srv = hs.Server(slots=1)
    for r in reqs:
        t, x = srv.submit(r[0], r[1], r[2], r[3], factor_key=r[4])
        st = srv.wait(t)
        assert st.done and st.error_code == 0
        _check(r, x)
        alone.append(x.copy())
    s1 = srv.stats()
    assert s1.peak_running == 1 and s1.completed == len(reqs)
    srv.close()

    srv = hs.Server(slots=4)
    tickets = [srv.submit(r[0], r[1], r[2], r[3], factor_key=r[4]) for r in reqs]  # all queued at once
    for (t, x), r, xa in zip(tickets, reqs, alone):
        st = srv.wait(t)
        assert st.error_code == 0 and st.relres <= RES_TOL
        assert st.t_arrival <= st.t_admit <= st.t_done
        _check(r, x)
        err = np.linalg.norm(x - xa) / np.linalg.norm(xa)
        assert err <= ERR_TOL, err
    s = srv.stats()
    assert s.completed == len(reqs) and s.failed == 0 and s.rejected == 0
    assert s.peak_running > 1  # requests overlapped on the device
    assert s.factor_hits >= 1  # repeat right-hand sides used resident factors
    assert 0 < s.latency_p50 <= s.latency_p99 <= s.latency_max
    srv.close()


def test_admission_follows_the_device_budget():
    reqs = _requests(count=8, seed=5)
    # a budget smaller than any request: rejected on submit
    srv = hs.Server(slots=4, hbm_budget=1)
    t, _ = srv.submit(reqs[0][0], reqs[0][1], reqs[0][2], reqs[0][3])
    st = srv.wait(t, check=False)
    assert st.error_code == 5  # memory: larger than the whole budget, rejected on submit
    srv.close()
    # a budget of a few requests: they queue for memory, and all complete
    srv = hs.Server(slots=4, hbm_budget=600 << 20)
    out = [srv.submit(r[0], r[1], r[2], r[3]) for r in reqs]
    for (t, x), r in zip(out, reqs):
        st = srv.wait(t)
        assert st.footprint <= 600 << 20
        _check(r, x)
    s = srv.stats()
    assert s.completed == len(reqs)
    srv.close()


def test_band_above_the_largest_tile_is_rejected():
    rp, ci, a, xt, b = hs.gen_banded(5000, 140, 140, 1.5, seed=3)
    srv = hs.Server(slots=2)
    t, _ = srv.submit(rp, ci, a, b)
    st = srv.wait(t, check=False)
    assert st.done and hs.ERR_NAMES[st.error_code] == "bandwidth"
    assert srv.stats().rejected == 1
    srv.close()


def test_a_full_queue_turns_requests_away_at_once():
    # load shedding: with max_queue waiting requests, the next one is completed
    # at once with SPIKE_ERR_BUSY; requests already queued still finish, and
    # poll() reports status without waiting
    srv = hs.Server(slots=1, max_queue=2)
    try:
        rp, ci, a, xt, b = hs.gen_banded(300_000, 64, 64, 1.5, seed=77, nrhs=4)
        tickets = [srv.submit(rp, ci, a, b, bandwidth=64) for _ in range(12)]  # no pattern scan: quick submits
        sts = [srv.poll(t) for t, _ in tickets]
        busy = [s for s in sts if s.done and hs.ERR_NAMES[s.error_code] == "busy"]
        assert len(busy) >= 12 - 1 - 2 - 2  # one running, two queued, slack for requests done meanwhile
        srv.drain()
        st = srv.stats()
        assert st.rejected_busy == len([1 for t, _ in tickets if hs.ERR_NAMES[srv.poll(t).error_code] == "busy"])
        assert st.completed + st.rejected_busy == 12 and st.completed >= 1
        for t, x in tickets:
            s = srv.poll(t)
            assert s.done
            if s.error_code == 0:
                assert s.relres <= RES_TOL and np.linalg.norm(x - xt) / np.linalg.norm(xt) <= 1e-10
    finally:
        srv.close()
