"""The serving loop (bl_server): continuous batching of whole jobs over memory slots."""
import time

import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _job(cfg, count):
    s = bl.SolidSys(cfg["lines"])
    phi, theta, gamma, w = (np.asarray(x)[:count] for x in cfg["powder"])
    pw = bl.powder.from_arrays(theta, phi, gamma, w)
    return dict(sys=s, pw=pw, ro=s.op(cfg["rho"]), det=s.op(cfg["det"]), npts=cfg["npts"], sw=cfg["sw"],
                wr=cfg["wr"], rotb=cfg["rotb"])


def _wait(srv, tickets, timeout=120.0):
    out, t0 = {}, time.time()
    while len(out) < len(tickets):
        for t in tickets:
            if t in out:
                continue
            st, fid, sw, lat = srv.result(t)
            if st >= srv.DONE:
                out[t] = (st, fid, lat)
        assert time.time() - t0 < timeout, "serving loop timed out"
        time.sleep(0.002)
    return out


def test_result_is_the_same_alone_and_in_the_mix():
    # 6 lanes over 12 GiB: 2 GiB grants, so the larger c3 systems run in several batches
    srv = bl.Server(0, lanes=6, pool_bytes=12 << 30)
    probe = _job(W.config(1), 128)
    t = srv.submit(**probe)
    alone = _wait(srv, [t])[t][1]
    mix = [_job(W.config(3, i), 96) for i in range(24)]
    tickets = []
    for i, j in enumerate(mix):
        tickets.append(srv.submit(**j))
        if i == 11:
            tp = srv.submit(**probe)
    res = _wait(srv, tickets + [tp])
    assert all(r[0] == srv.DONE for r in res.values())
    np.testing.assert_array_equal(res[tp][1], alone)
    # and equal to the direct (non-served) call
    direct = bl.oneFID(probe["sys"], probe["npts"], probe["sw"], probe["wr"], probe["rotb"]).FID(
        probe["pw"], probe["ro"], probe["det"])
    np.testing.assert_array_equal(alone, direct)
    q, r, d, fl = srv.stats()
    assert q == 0 and r == 0 and d >= 26 and fl > 0
    srv.close()


def test_cancel_queued_and_reject_oversized():
    srv = bl.Server(0, lanes=1, pool_bytes=64 << 20)
    j = _job(W.config(0), 64)
    tickets = [srv.submit(**j) for _ in range(6)]
    srv.cancel(tickets[-1])  # still queued behind five jobs on one lane
    res = _wait(srv, tickets[:-1])
    assert all(r[0] == srv.DONE for r in res.values())
    st, fid, _, _ = srv.result(tickets[-1])
    assert st == srv.CANCELLED and fid is None
    big = _job(dict(W.config(1), sw=2000 * 20e3), 64)  # one warp needs > 64 MiB
    tb = srv.submit(**big)  # queued; the planner fails it
    with pytest.raises(bl.BlochError) as e:
        _wait(srv, [tb])
    assert "MiB" in str(e.value)
    srv.close()


def test_admission_waits_for_memory():
    """Two lanes but a pool that holds one grant: jobs run one at a time, all complete,
    results equal the direct call."""
    cfg = W.config(3, 0)
    j = _job(cfg, 64)
    lo, hi = bl.job_bytes(**j)
    srv = bl.Server(0, lanes=2, pool_bytes=int(lo * 1.5))
    tickets = [srv.submit(**j) for _ in range(3)]
    res = _wait(srv, tickets, timeout=300)
    assert all(r[0] == srv.DONE for r in res.values())
    direct = bl.oneFID(j["sys"], j["npts"], j["sw"], j["wr"], j["rotb"]).FID(j["pw"], j["ro"], j["det"])
    for t in tickets:
        np.testing.assert_array_equal(res[t][1], direct)
    srv.close()


def test_point_to_point_requests_are_served():
    """A point-to-point request (with an rf schedule) through the serving loop, among ordinary
    ones, gives the direct p2pFID result bit for bit."""
    srv = bl.Server(0, lanes=4, pool_bytes=8 << 30)
    j = _job(W.config(1), 192)
    sched = [(0, "1H", 60000.0, 0.0, 0.0), (2, "1H", 60000.0, 90.0, 500.0)]
    args = dict(sys=j["sys"], pw=j["pw"], ro=j["ro"], det=j["det"], npts=300, wr=j["wr"], rotb=j["rotb"],
                base=4, factor=3, maxtstep=3e-6, rf_chunks=sched)
    others = [srv.submit(**_job(W.config(3, i), 64)) for i in range(6)]
    t = srv.submit_p2p(**args)
    res = _wait(srv, others + [t])
    assert all(r[0] == srv.DONE for r in res.values())
    direct = bl.oneFID(j["sys"], 300, 0.0, j["wr"], j["rotb"]).p2pFID(j["pw"], j["ro"], j["det"], 4, 3, 3e-6,
                                                                      rf_chunks=sched)
    np.testing.assert_array_equal(res[t][1], direct)
    srv.close()


def test_mixed_result_is_the_same_alone_and_in_the_mix():
    """The form the target measures: a mixed-precision request (6 x 1H: its blocks of 15 and
    20 run on the tensor-core step and Dyson kernels) gives the same FID bit for bit alone and
    among mixed and FP64 requests of other systems, within 1e-6 of its FP64 result."""
    srv = bl.Server(0, lanes=6, pool_bytes=12 << 30)
    probe = _job(W.config(3, 2), 64)
    t = srv.submit(**probe, precision=1, step_method="taylor")
    alone = _wait(srv, [t])[t][1]
    tickets = []
    for i in range(16):
        tickets.append(srv.submit(**_job(W.config(3, 100 + i), 64), precision=i % 2, step_method="taylor"))
        if i == 7:
            tp = srv.submit(**probe, precision=1, step_method="taylor")
    tf = srv.submit(**probe, precision=0, step_method="taylor")
    res = _wait(srv, tickets + [tp, tf], timeout=300)
    assert all(r[0] == srv.DONE for r in res.values())
    np.testing.assert_array_equal(res[tp][1], alone)
    err = np.linalg.norm(alone - res[tf][1]) / np.linalg.norm(res[tf][1])
    assert 0 < err <= 1e-6, err
    srv.close()


def test_small_requests_pass_a_blocked_large_head():
    """Bounded skip-ahead: a pool that holds one large job's grant (its one-warp size, so it
    runs in many batches) plus one small job.  With the first large job running, the second
    waits at the head of the queue; the small jobs behind it are admitted on the other lane
    and finish long before the first large job does.  Results equal the direct call."""
    big = _job(W.config(1), 3722)
    lo, hi = bl.job_bytes(**big)
    small = _job(W.config(0), 64)
    slo, shi = bl.job_bytes(**small)
    pool = lo + shi + (1 << 20)  # < 2 lo: one large grant at a time; share = pool / 2 < lo
    assert pool < 2 * lo
    srv = bl.Server(0, lanes=2, pool_bytes=int(pool))
    ta = srv.submit(**big)
    tb = srv.submit(**big)
    ts = [srv.submit(**small) for _ in range(4)]
    res = _wait(srv, [ta, tb] + ts, timeout=600)
    assert all(r[0] == srv.DONE for r in res.values())
    lat_a = res[ta][2]
    assert max(res[t][2] for t in ts) < lat_a, (lat_a, [res[t][2] for t in ts])
    np.testing.assert_array_equal(res[ta][1], res[tb][1])
    direct = bl.oneFID(small["sys"], small["npts"], small["sw"], small["wr"], small["rotb"]).FID(
        small["pw"], small["ro"], small["det"])
    for t in ts:
        np.testing.assert_array_equal(res[t][1], direct)
    srv.close()


def test_tensor_core_request_is_the_same_alone_and_in_the_mix():
    """A c2-sized mixed request (8 x 1H: its blocks 56 and 70 run on the tensor-core step and
    Dyson kernels) gives the direct call's FID bit for bit, alone and among other requests
    running on the other lanes."""
    srv = bl.Server(0, lanes=4, pool_bytes=24 << 30)
    probe = _job(W.config(2), 32)
    t = srv.submit(**probe, precision=1, step_method="taylor")
    alone = _wait(srv, [t], timeout=300)[t][1]
    others = [srv.submit(**_job(W.config(3, 200 + i), 64), precision=i % 2, step_method="taylor") for i in range(6)]
    tp = srv.submit(**probe, precision=1, step_method="taylor")
    res = _wait(srv, others + [tp], timeout=300)
    assert all(r[0] == srv.DONE for r in res.values())
    np.testing.assert_array_equal(res[tp][1], alone)
    direct = bl.oneFID(probe["sys"], probe["npts"], probe["sw"], probe["wr"], probe["rotb"], precision=1,
                       step_method="taylor").FID(probe["pw"], probe["ro"], probe["det"])
    np.testing.assert_array_equal(alone, direct)
    srv.close()
