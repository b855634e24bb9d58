"""The allocation-free entry point, bl_powder_fid_noalloc, through the C ABI.

It serves callers that may not allocate device memory during a call (a host program that
claims the GPU's memory itself, or a timing-critical loop where cudaMalloc/cudaFree and
their device-wide synchronisation are off limits).  It must give the same FID as
bl_powder_fid, call after call, although every call reuses the same static device array.
This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W
from helpers import rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _inputs(cfg, count=None):
    s = bl.SolidSys(cfg["lines"])
    phi, theta, gamma, w = (np.asarray(x) for x in cfg["powder"])
    if count:
        phi, theta, gamma, w = phi[:count], theta[:count], gamma[:count], w[:count]
    pw = bl.powder.from_arrays(theta, phi, gamma, w)
    ro = np.ascontiguousarray(s.op(cfg["rho"]))
    det = np.ascontiguousarray(s.op(cfg["det"]))
    params = bl.FidParams(cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], 0.0, 0, 0)
    return s, pw, ro, det, params


def _call(fn, ctx, s, pw, ro, det, params, npts):
    out = np.zeros(npts, dtype=np.complex128)
    sw = ctypes.c_double()
    st = fn(ctx._h, s._h, pw._h, ro.ctypes.data, det.ctypes.data, ctypes.byref(params), out.ctypes.data,
            ctypes.byref(sw))
    return st, out, sw.value


@pytest.mark.parametrize("cfg,count", [(W.config(0), None), (W.config(1), 200)],
                         ids=["c0_full_powder", "c1_200_crystallites_batched"])
def test_noalloc_matches_allocating_entry_point_twice(cfg, count):
    lib = bl.load()
    ctx = bl.Context(0)
    s, pw, ro, det, params = _inputs(cfg, count)
    st, ref, sw_ref = _call(lib.bl_powder_fid, ctx, s, pw, ro, det, params, cfg["npts"])
    assert st == 0, lib.bl_last_error()
    for _ in range(2):  # the second call runs on the first call's leftover scratch contents
        st, fid, sw = _call(lib.bl_powder_fid_noalloc, ctx, s, pw, ro, det, params, cfg["npts"])
        assert st == 0, lib.bl_last_error()
        assert sw == sw_ref
        assert rel(fid, ref) <= TOL, rel(fid, ref)


def test_noalloc_mixed_form_matches_allocating_entry_point():
    """The mixed form (double-float step and Dyson, single-precision stages) through the
    static scratch, in batches, gives bl_powder_fid's result."""
    lib = bl.load()
    ctx = bl.Context(0)
    cfg = W.config(1)
    s, pw, ro, det, _ = _inputs(cfg, 200)
    params = bl.FidParams(cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], 0.0, 1, 1)
    st, ref, _ = _call(lib.bl_powder_fid, ctx, s, pw, ro, det, params, cfg["npts"])
    assert st == 0, lib.bl_last_error()
    st, fid, _ = _call(lib.bl_powder_fid_noalloc, ctx, s, pw, ro, det, params, cfg["npts"])
    assert st == 0, lib.bl_last_error()
    assert rel(fid, ref) <= TOL, rel(fid, ref)


def test_noalloc_rejects_a_job_beyond_its_scratch():
    lib = bl.load()
    ctx = bl.Context(0)
    cfg = dict(W.config(1), sw=2000 * 20e3)  # 2000 steps per period: one warp needs >64 MiB
    s, pw, ro, det, params = _inputs(cfg, 64)
    st, _, _ = _call(lib.bl_powder_fid_noalloc, ctx, s, pw, ro, det, params, cfg["npts"])
    assert st == 4
    assert b"static device scratch" in lib.bl_last_error()
