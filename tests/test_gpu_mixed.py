"""The mixed-precision form (precision=1): step exponential and Dyson product in double-float
(hi + lo floats) on the FP32 pipe, Floquet eigen-decomposition and powder sum in FP64;
eigenframe, Q/R, Fave and FID reconstruction in single precision.  Gate: <= 1e-6 relative L2
FID error against the FP64 path and the reference."""
import numpy as np
import pytest

from blochlib_gb300 import workloads as W
from helpers import gpu_fid, golden_cases, load_golden, rel

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-6


@pytest.mark.parametrize("case", [c for c in golden_cases() if not c.startswith("static")])
def test_mixed_matches_reference_golden(case):
    job, rows, fid64, _, sw = load_golden(case)
    fid, sw_m = gpu_fid(job, rows, return_sw=True, precision=1, step_method="taylor")
    assert sw_m == sw
    assert rel(fid, fid64) <= TOL_MIXED, rel(fid, fid64)


@pytest.mark.parametrize("cfg_index,count", [(0, 1154), (1, 512), (2, 32)])
def test_mixed_vs_fp64_on_configs(cfg_index, count):
    cfg = W.config(cfg_index)
    rows = np.stack(cfg["powder"], axis=1)[:count]
    job = W.job_text(cfg)
    f64 = gpu_fid(job, rows, precision=0, step_method="taylor")
    fmx = gpu_fid(job, rows, precision=1, step_method="taylor")
    err = rel(fmx, f64)
    assert err <= TOL_MIXED, err
    assert err > 0  # the single-precision stages really ran


def test_mixed_results_state_their_error():
    """error_sample: the mixed FID states its error against FP64 on a sample of crystallites,
    through bl_powder_fid and through the serving loop; the statement is of the size of the
    result's actual error (c1, 512 crystallites: both ~1e-8, under the 1e-6 bar)."""
    import blochlib_gb300 as bl
    cfg = W.config(1)
    rows = np.stack(cfg["powder"], axis=1)[:512]
    job = W.job_text(cfg)
    f64 = gpu_fid(job, rows, precision=0, step_method="taylor")
    s = bl.SolidSys(cfg["lines"])
    pw = bl.powder.from_arrays(rows[:, 1], rows[:, 0], rows[:, 2], rows[:, 3])
    drv = bl.oneFID(s, cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], precision=1, step_method="taylor",
                    error_sample=32)
    fmx = drv.FID(pw, s.op(cfg["rho"]), s.op(cfg["det"]))
    actual = rel(fmx, f64)
    stated = drv.error_statement
    assert stated is not None and 0 < stated <= TOL_MIXED, stated
    assert actual / 30 <= stated <= actual * 30, (stated, actual)
    # an FP64 result states nothing
    plain = bl.oneFID(s, cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], precision=0, error_sample=32)
    plain.FID(pw, s.op(cfg["rho"]), s.op(cfg["det"]))
    assert plain.error_statement is None
    srv = bl.Server(0, lanes=2, pool_bytes=4 << 30)
    t = srv.submit(sys=s, pw=pw, ro=s.op(cfg["rho"]), det=s.op(cfg["det"]), npts=cfg["npts"], sw=cfg["sw"],
                   wr=cfg["wr"], rotb=cfg["rotb"], precision=1, step_method="taylor", error_sample=32)
    import time
    t0 = time.time()
    while True:
        st, fid, _, _ = srv.result(t)
        if st >= srv.DONE:
            break
        assert time.time() - t0 < 120
        time.sleep(0.002)
    assert st == srv.DONE
    np.testing.assert_array_equal(fid, fmx)
    assert srv.last_error_statement == stated
    srv.close()
