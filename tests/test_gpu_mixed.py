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
