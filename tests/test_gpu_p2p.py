"""Point-to-point FIDs (bl_p2p_fid) on the GPU against the oracle's direct propagation.

The reference forms each dwell propagator from chunk products (PropReduce, examples/qmsims/
MMMQMAS/propreduce.cc) and steps rho point by point; the engine takes one rotor period of
Dyson products and the Floquet phases instead.  Tolerance: <= 1e-10 relative L2 (FP64), as
for the gamma-COMPUTE FID; the mixed form <= 1e-6."""
import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W
from helpers import gpu_fid, oracle_fid, parse_job, rel
from test_gpu_parity import big_system, quad2_system, random_system

pytestmark = pytest.mark.gpu
TOL = 1e-10


def as_p2p(job, rng, base=None, factor=None, maxtstep=None):
    """The job with a p2p line: a rotor period in `base` chunks, a point every `factor`."""
    lines, kv = parse_job(job)
    base = int(rng.integers(1, 10)) if base is None else base
    factor = int(rng.integers(1, 12)) if factor is None else factor
    wr = float(kv["wr"])
    if maxtstep is None:
        maxtstep = float(rng.choice([0.0, 0.3, 0.7])) / (wr * base) if wr else 0.0
    return job + f"p2p: {base} {factor}\nmaxtstep: {maxtstep!r}\n"


@pytest.mark.parametrize("method", ["eigh", "taylor"])
@pytest.mark.parametrize("seed", range(12))
def test_p2p_random_systems_match_oracle(seed, method):
    """Homo/heteronuclear and quadrupolar systems, rho symmetric or not, random base/factor
    (either larger) and chunk step counts."""
    rng = np.random.default_rng(500 + seed)
    job, rows = random_system(seed)
    job = as_p2p(job, rng)
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method=method)
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.parametrize("seed", range(6))
def test_p2p_second_order_quadrupole_matches_oracle(seed):
    rng = np.random.default_rng(700 + seed)
    job, rows = quad2_system(seed)
    job = as_p2p(job, rng)
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method="taylor")
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.parametrize("seed,nspin,rho,det", [(0, 5, "Fx", "Fp"), (1, 5, "Fx+Fz", "Fp"), (2, 6, "Ix 0", "Ix 0")])
def test_p2p_big_blocks_match_oracle(seed, nspin, rho, det):
    rng = np.random.default_rng(900 + seed)
    job, rows = big_system(seed, nspin, rho, det)
    job = as_p2p(job, rng, base=int(rng.integers(2, 6)), factor=int(rng.integers(1, 8)))
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method="taylor")
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.parametrize("seed,nspin", [(0, 5), (2, 6)])
def test_p2p_big_blocks_mixed_within_1e6(seed, nspin):
    """The mixed form's large-block kernels (double-float step and Dyson, FP32 sweeps over K)
    on the point-to-point path, with a chunk rf schedule on top: <= 1e-6 against the oracle."""
    rng = np.random.default_rng(950 + seed)
    job, rows = big_system(seed, nspin, "Fx", "Fp")
    b = int(rng.integers(2, 6))
    job = as_p2p(job, rng, base=b, factor=int(rng.integers(1, 8)))
    job += f"rfc: {int(rng.integers(0, b))} 1H {rng.uniform(1e4, 5e4):.9g} 0 0\n"
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, step_method="taylor", precision=1)
    assert 0 < rel(fid, ref) <= 1e-6, rel(fid, ref)


def test_p2p_gcd_reduction():
    """PropReduce divides base and factor by their gcd: (12, 8) is (3, 2)."""
    rng = np.random.default_rng(3)
    job, rows = random_system(4)
    a = gpu_fid(as_p2p(job, rng, 12, 8, 0.0), rows)
    b = gpu_fid(as_p2p(job, rng, 3, 2, 0.0), rows)
    np.testing.assert_array_equal(a, b)


def test_p2p_mixed_within_1e6():
    cfg = W.config(1)
    rows = np.stack(cfg["powder"], axis=1)[:256]
    job = W.job_text(dict(cfg, npts=512)) + "p2p: 9 7\nmaxtstep: 2e-06\n"
    f64 = gpu_fid(job, rows, step_method="taylor")
    mix = gpu_fid(job, rows, step_method="taylor", precision=1)
    assert rel(mix, f64) <= 1e-6, rel(mix, f64)


def test_p2p_full_powder_first_point():
    """c1's full powder (3722 crystallites), dwell 7/9 of a period: point 0 is
    sum_c w_c Tr(rho det) / Tr(det det^H) exactly, whatever the propagators."""
    cfg = W.config(1)
    rows = np.stack(cfg["powder"], axis=1)
    job = W.job_text(cfg) + "p2p: 9 7\nmaxtstep: 2e-06\n"
    fid = gpu_fid(job, rows, step_method="taylor")
    lines, kv = parse_job(job)
    s = bl.SolidSys(lines)
    ro, det = s.op(kv["rho"]), s.op(kv["det"])
    want = np.trace(ro @ det) / np.sum(np.abs(det) ** 2) * rows[:, 3].sum()
    assert abs(fid[0] - want) <= 1e-12 * abs(want)
    assert np.all(np.isfinite(fid))


def test_p2p_rejects_bad_parameters():
    job, rows = random_system(0)
    lines, kv = parse_job(job)
    s = bl.SolidSys(lines)
    pw = bl.powder.from_arrays(theta=rows[:, 1], phi=rows[:, 0], gamma=rows[:, 2], weight=rows[:, 3])
    drv = bl.oneFID(s, 16, float(kv["sw"]), float(kv["wr"]), float(kv["rotb"]))
    with pytest.raises(bl.BlochError):
        drv.p2pFID(pw, s.op("Fx"), s.op("Fp"), 0, 1)
    with pytest.raises(bl.BlochError):
        drv.p2pFID(pw, s.op("Fx"), s.op("Fp"), 3, -2)
    # more than 16384 steps per rotor period
    with pytest.raises(bl.BlochError):
        drv.p2pFID(pw, s.op("Fx"), s.op("Fp"), 64, 1, maxtstep=1e-3 / (float(kv["wr"]) * 64 * 300))
