"""Continuous rf during the FID (SolidSys.addRf / bl_system_add_rf): GPU against the oracle.

The oracle adds solid-2.0's PulseData::Pulse term to H in the lab frame (complex H); the
engine keeps H real and carries a phase off the x axis in the frame exp(-i phase Fz_iso),
so these tests check that transformation as well.  Tolerance <= 1e-10 relative (FP64)."""
import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W
from helpers import gpu_fid, oracle_fid, parse_job, rel
from test_gpu_parity import random_system

TOL = 1e-10


def with_rf(job, rng, nfields=None):
    lines, kv = parse_job(job)
    isos = sorted({l.split()[1] for l in lines if l.startswith("T ")})
    out = job
    for _ in range(int(rng.integers(1, 3)) if nfields is None else nfields):
        iso = str(rng.choice(isos))
        phase = float(rng.choice([0.0, 90.0, 180.0, 270.0, rng.uniform(0, 360)]))
        out += f"rf: {iso} {rng.uniform(5e3, 1e5):.9g} {phase:.9g} {rng.uniform(-5e3, 5e3):.9g}\n"
    return out


def strong_hetero_j(job):
    """A strong J between different isotopes: an off-x rf phase is then refused."""
    lines, _ = parse_job(job)
    iso = {int(l.split()[2]): l.split()[1] for l in lines if l.startswith("T ")}
    for l in lines:
        t = l.split()
        if t[0] == "J" and len(t) >= 5 and t[4] == "1" and iso[int(t[2])] != iso[int(t[3])]:
            return True
    return False


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["eigh", "taylor"])
@pytest.mark.parametrize("seed", range(12))
def test_rf_random_systems_match_oracle(seed, method):
    rng = np.random.default_rng(1300 + seed)
    job, rows = random_system(seed)
    job = with_rf(job, rng)
    if seed % 3 == 2:  # and the point-to-point form
        job += f"p2p: {int(rng.integers(1, 7))} {int(rng.integers(1, 7))}\nmaxtstep: 3e-06\n"
    if strong_hetero_j(job) and any(float(l.split()[3]) % 180 for l in job.splitlines() if l.startswith("rf:")):
        pytest.skip("off-x phase with a strong heteronuclear J: refused (see test_rf_frame_refused)")
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method=method)
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.gpu
def test_rf_spin_lock_mixed_within_1e6():
    """c1 (4 1H) under a 1H spin-lock: one Fz-mixing block of 16, mixed form vs FP64."""
    cfg = W.config(1)
    rows = np.stack(cfg["powder"], axis=1)[:256]
    job = W.job_text(dict(cfg, npts=512)) + "rf: 1H 50000 30 0\n"
    f64 = gpu_fid(job, rows, step_method="taylor")
    mix = gpu_fid(job, rows, step_method="taylor", precision=1)
    assert rel(mix, f64) <= 1e-6, rel(mix, f64)
    ref, _ = oracle_fid(job, rows[:16])
    assert rel(gpu_fid(job, rows[:16], step_method="taylor"), ref) <= TOL


def test_rf_frame_refused():
    """An off-x phase needs H to commute with the isotope's Fz; a strong 13C-1H J does not."""
    s = bl.SolidSys(["numspin 2", "T 13C 0", "T 1H 1", "J 120 0 1 1", "D 5000 0 1 0 30 0"])
    s.addRf("1H", 50000, 0.0)      # x phase: no frame needed
    s.addRf("1H", 20000, 180.0)    # -x: still real
    with pytest.raises(bl.BlochError):
        s.addRf("1H", 20000, 45.0)
    assert max(s.blocks()) == 4     # the x fields join the 1H sectors with the strong J


def test_rf_joins_blocks():
    s = bl.SolidSys(["numspin 3", "T 1H 0", "T 1H 1", "T 13C 2", "D 9000 0 1 0 30 0"])
    before = sorted(s.blocks())
    s.addRf("1H", 40000, 60.0, 1000.0)
    assert max(s.blocks()) > max(before)
    s2 = bl.SolidSys(["numspin 2", "T 1H 0", "T 13C 1"])
    s2.addRf("1H", 0.0, 90.0, 5000.0)  # amp 0: nothing at all, the offset included
    assert sorted(s2.blocks()) == [1, 1, 1, 1]


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["eigh", "taylor"])
@pytest.mark.parametrize("seed", range(10))
def test_rf_schedule_random_systems_match_oracle(seed, method):
    """rf changing within the rotor period (p2p): random chunk schedules of 1-3 fields with
    any phase, on top of random continuous fields, against the oracle."""
    rng = np.random.default_rng(1700 + seed)
    job, rows = random_system(seed)
    if seed % 2:
        job = with_rf(job, rng, nfields=1)
    lines, kv = parse_job(job)
    isos = sorted({l.split()[1] for l in lines if l.startswith("T ")})
    b, f = int(rng.integers(2, 7)), int(rng.integers(1, 7))
    job += f"p2p: {b} {f}\nmaxtstep: {0.4 / (float(kv['wr']) * b)!r}\n"
    for _ in range(int(rng.integers(1, 4))):
        job += (f"rfc: {int(rng.integers(0, b))} {rng.choice(isos)} {rng.uniform(1e4, 9e4):.9g} "
                f"{rng.uniform(0, 360):.9g} {rng.uniform(-3e3, 3e3):.9g}\n")
    if strong_hetero_j(job):
        pytest.skip("off-x phases with a strong heteronuclear J: refused")
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method=method)
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.gpu
def test_rf_schedule_needs_p2p():
    s = bl.SolidSys(["numspin 2", "T 13C 0", "T 1H 1", "D 5000 0 1 0 30 0"])
    with pytest.raises(bl.BlochError, match="needs spinning"):  # the static branch takes no schedule
        bl.Job.p2p(s, bl.powder(bl.powder.zcw, 21, 8), s.op("Ix 0"), s.op("Ip 0"), 16, 0.0, 54.7356, 3, 2,
                   sw=1e5, rf_chunks=[(0, "1H", 5e4, 0.0, 0.0)])
