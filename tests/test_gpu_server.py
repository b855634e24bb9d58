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
