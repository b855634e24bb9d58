"""CUDA engine vs the reference (golden fixtures) and vs the CPU oracle, through the C ABI.

Tolerance: the plain FP64 path must reproduce the reference's FP64 FID to <= 1e-10
relative L2 error (||fid - ref|| / ||ref||)."""
import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W
from helpers import gpu_fid, golden_cases, load_golden, oracle_fid, parse_job, rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("method,fave", [("eigh", "fft"), ("taylor", "fft"), ("eigh", "direct")])
@pytest.mark.parametrize("case", golden_cases())
def test_gpu_matches_reference_golden(case, method, fave):
    job, rows, fid64, fid32, sw = load_golden(case)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method=method, fave_method=fave)
    assert sw_g == sw
    assert rel(fid, fid64) <= TOL, rel(fid, fid64)


def random_system(seed):
    rng = np.random.default_rng(seed)
    kind = seed % 3
    if kind == 0:   # homonuclear 1H, 2-4 spins
        n = int(rng.integers(2, 5))
        iso = ["1H"] * n
    elif kind == 1:  # heteronuclear mix
        n = int(rng.integers(2, 5))
        iso = [str(rng.choice(["1H", "13C", "15N"])) for _ in range(n)]
    else:            # spin-1 quadrupole with protons
        n = int(rng.integers(2, 4))
        iso = ["2H"] + ["1H"] * (n - 1)
    lines = [f"numspin {n}"] + [f"T {iso[k]} {k}" for k in range(n)]
    for k in range(n):
        a = rng.uniform(0, 360, 3)
        lines.append(f"C {rng.uniform(-3e3, 3e3):.9g} {rng.uniform(-8e3, 8e3):.9g} {rng.uniform(0, 1):.9g} {k} "
                     f"{a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    for i in range(n):
        for j in range(i + 1, n):
            a = rng.uniform(0, 360, 3)
            lines.append(f"D {rng.uniform(-2e4, 2e4):.9g} {i} {j} {a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
            if rng.uniform() < 0.5:
                lines.append(f"J {rng.uniform(0, 200):.9g} {i} {j} {int(rng.uniform() < 0.3)}")
    if kind == 2:
        a = rng.uniform(0, 360, 3)
        lines.append(f"Q {rng.uniform(5e4, 2e5):.9g} {rng.uniform(0, 1):.9g} 0 {a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    rho, det = [("Fx", "Fp"), ("Fx+Fz", "Fp"), ("Ix 0", "Ix 0"), ("Iy 0", "Ip 0")][seed % 4]
    wr = float(rng.uniform(5e3, 30e3))
    n_steps = int(rng.integers(12, 70))
    job = "\n".join(f"spin: {l}" for l in lines) + (
        f"\nnpts: {int(rng.integers(50, 300))}\nsw: {n_steps * wr!r}\nwr: {wr!r}\nrotb: {rng.uniform(30, 70)!r}\n"
        f"rho: {rho}\ndet: {det}\n")
    c = int(rng.integers(1, 40))
    rows = np.stack([rng.uniform(0, 2 * np.pi, c), np.arccos(rng.uniform(-1, 1, c)), rng.uniform(0, 2 * np.pi, c),
                     rng.uniform(0.1, 1, c)], axis=1)
    return job, rows


@pytest.mark.parametrize("method,fave", [("eigh", "fft"), ("taylor", "fft"), ("taylor", "direct")])
@pytest.mark.parametrize("seed", range(12))
def test_gpu_matches_oracle_random_systems(seed, method, fave):
    job, rows = random_system(seed)
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method=method, fave_method=fave)
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.parametrize("method", ["eigh", "taylor"])
def test_c0_full_powder_matches_oracle(method):
    cfg = W.config(0)
    job = W.job_text(cfg)
    rows = np.stack(cfg["powder"], axis=1)
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, step_method=method)
    assert rel(fid, ref) <= TOL, rel(fid, ref)


def _c1_job(count=None):
    cfg = W.config(1)
    rows = np.stack(cfg["powder"], axis=1)
    if count:
        rows = rows[:count]
    return W.job_text(cfg), rows


def test_batched_run_is_bitwise_identical_to_single_batch():
    """Several batches (the one-shot call batches inside the context's kept region) equal one
    batch bit for bit; a second call reuses the region, a resident job on the context takes
    the region back, and the next one-shot call builds it again."""
    job, rows = _c1_job(200)
    one = gpu_fid(job, rows)
    small = bl.Context(0, hbm_budget=40 << 20)  # forces several crystallite batches
    many = gpu_fid(job, rows, ctx=small)
    np.testing.assert_array_equal(one, many)
    np.testing.assert_array_equal(gpu_fid(job, rows, ctx=small), one)
    lines, kv = parse_job(job)
    s = bl.SolidSys(lines)
    pw = bl.powder.from_arrays(theta=rows[:, 1], phi=rows[:, 0], gamma=rows[:, 2], weight=rows[:, 3])
    res = bl.Job(s, pw, s.op(kv["rho"]), s.op(kv["det"]), int(kv["npts"]), float(kv["sw"]), float(kv["wr"]),
                 float(kv["rotb"]), ctx=small)
    res.run()
    np.testing.assert_array_equal(res.read(), one)
    res.close()
    np.testing.assert_array_equal(gpu_fid(job, rows, ctx=small), one)


def test_crystallite_alone_equals_crystallite_in_batch():
    job, rows = _c1_job(96)
    c = 37
    alone = gpu_fid(job, rows[c:c + 1])
    masked = rows.copy()
    masked[:, 3] = 0.0
    masked[c, 3] = rows[c, 3]
    inbatch = gpu_fid(job, masked)
    np.testing.assert_array_equal(alone, inbatch)


def test_c1_full_size_properties():
    """Full c1 (3722 crystallites, 2048 points): size-independent checks."""
    job, rows = _c1_job()
    full = gpu_fid(job, rows)
    # rho = Fx = (D + D^H)/2 with D = F+ (D^2 = 0): fid[0] = 2 Tr(D D^H) sum(w)
    lines, kv = parse_job(job)
    s = bl.SolidSys(lines)
    D = s.op("Fp")
    expect0 = 2 * np.trace(D @ D.conj().T).real * rows[:, 3].sum()
    assert abs(full[0] - expect0) <= 1e-12 * abs(expect0)
    # linearity in the powder weights: two halves sum to the whole
    a, b = rows.copy(), rows.copy()
    a[1861:, 3] = 0.0
    b[:1861, 3] = 0.0
    assert rel(gpu_fid(job, a) + gpu_fid(job, b), full) <= 1e-13
    # the first 8 crystallites against the oracle
    ref8, _ = oracle_fid(job, rows[:8])
    assert rel(gpu_fid(job, rows[:8]), ref8) <= TOL


def test_unsupported_inputs_return_status():
    cfg = W.config(0)
    rows = np.stack(cfg["powder"], axis=1)[:4]
    # 13 spins 1/2: dimension 8192 > 4096 (the largest block a SolidSys of dimension <= 4096
    # can have is 924, within the engine's 1024)
    big = "\n".join(f"spin: {l}" for l in ["numspin 13"] + [f"D -5000 {i} {i + 1}" for i in range(12)])
    big += "\nnpts: 16\nsw: 100000\nwr: 10000\nrotb: 54.7356\nrho: Fx\ndet: Fp\n"
    with pytest.raises(bl.BlochError) as e:
        gpu_fid(big, rows)
    assert e.value.status == 5
    too_slow = W.job_text(dict(cfg, sw=1000.0))  # sw/wr rounds to zero steps
    with pytest.raises(bl.BlochError) as e:
        gpu_fid(too_slow, rows)
    assert e.value.status == 1


@pytest.mark.parametrize("wr,rotb", [(0.0, 54.7356), (10000.0, 0.0), (0.0, 0.0)])
def test_static_powder_fid_matches_oracle(wr, rotb):
    """oneFID::FID takes the static branch when wr == 0 or the rotor angle is 0."""
    cfg = W.config(1)
    rows = np.stack(cfg["powder"], axis=1)[:40]
    job = W.job_text(dict(cfg, wr=wr, rotb=rotb, sw=250000.0, npts=700))
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True)
    assert sw_g == sw == 250000.0
    assert rel(fid, ref) <= TOL, rel(fid, ref)


def test_resident_job_reruns_identically():
    job, rows = _c1_job(64)
    lines, kv = parse_job(job)
    s = bl.SolidSys(lines)
    pw = bl.powder.from_arrays(rows[:, 1], rows[:, 0], rows[:, 2], rows[:, 3])
    j = bl.Job(s, pw, s.op(kv["rho"]), s.op(kv["det"]), int(kv["npts"]), float(kv["sw"]), float(kv["wr"]),
               float(kv["rotb"]))
    j.run()
    a = j.read()
    j.set_profiling(True)
    j.run()
    b = j.read()
    np.testing.assert_array_equal(a, b)
    st = j.stage_times()
    assert st["k_fave"][1] >= 1 and st["k_step_prop"][0] > 0
    assert j.launches >= 8


def big_system(seed, nspin, rho, det):
    rng = np.random.default_rng(1000 + seed)
    # one 13C among >= 5 protons still leaves proton blocks larger than 8
    iso = ["1H"] * nspin if (seed % 2 == 0 or nspin < 6) else ["1H"] * (nspin - 1) + ["13C"]
    lines = [f"numspin {nspin}"] + [f"T {iso[k]} {k}" for k in range(nspin)]
    for k in range(nspin):
        a = rng.uniform(0, 360, 3)
        lines.append(f"C {rng.uniform(-2e3, 2e3):.9g} {rng.uniform(-6e3, 6e3):.9g} {rng.uniform(0, 1):.9g} {k} "
                     f"{a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    for i in range(nspin):
        for j in range(i + 1, nspin):
            a = rng.uniform(0, 360, 3)
            lines.append(f"D {rng.uniform(-1.5e4, 1.5e4):.9g} {i} {j} {a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    lines.append("J 90 0 1 1")
    wr = float(rng.uniform(8e3, 30e3))
    n_steps = int(rng.integers(10, 40))
    job = "\n".join(f"spin: {l}" for l in lines) + (
        f"\nnpts: 300\nsw: {n_steps * wr!r}\nwr: {wr!r}\nrotb: {W.MAGIC_ANGLE!r}\nrho: {rho}\ndet: {det}\n")
    c = 2 if nspin < 7 else 1
    rows = np.stack([rng.uniform(0, 2 * np.pi, c), np.arccos(rng.uniform(-1, 1, c)), rng.uniform(0, 2 * np.pi, c),
                     rng.uniform(0.1, 1, c)], axis=1)
    return job, rows


@pytest.mark.parametrize("seed,nspin,rho,det", [(0, 5, "Fx", "Fp"), (1, 5, "Fx+Fz", "Fp"), (2, 6, "Ix 0", "Ix 0"),
                                                (3, 6, "Fx", "Fp"), (4, 7, "Fx", "Fp")])
def test_big_blocks_match_oracle(seed, nspin, rho, det):
    """Hamiltonian blocks larger than 8 (5-7 spins) run on the CTA-per-block kernels."""
    job, rows = big_system(seed, nspin, rho, det)
    lines, _ = parse_job(job)
    assert max(bl.SolidSys(lines).blocks()) > 8
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method="taylor")
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


@pytest.mark.parametrize("seed,nspin,rho,det", [(0, 5, "Fx", "Fp"), (3, 6, "Fx", "Fp"), (4, 7, "Fx", "Fp")])
def test_big_blocks_mixed_within_1e6(seed, nspin, rho, det):
    """The mixed form on the CTA-per-block kernels: step and Dyson in double-float, Floquet
    from the double-float A, eigenframe from its high parts; <= 1e-6 against the oracle."""
    job, rows = big_system(seed, nspin, rho, det)
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, step_method="taylor", precision=1)
    assert 0 < rel(fid, ref) <= 1e-6, rel(fid, ref)


def test_big_blocks_mixed_batch_invariant():
    """Each crystallite's double-float arithmetic is its own: one crystallite alone gives the
    bits it gets beside others."""
    job, rows = big_system(1, 6, "Fx", "Fp")
    rows = np.concatenate([rows, rows[::-1] * [1.1, 0.9, 1.05, 1.0]])
    both = gpu_fid(job, rows, step_method="taylor", precision=1)
    alone = gpu_fid(job, rows[:1], step_method="taylor", precision=1)
    masked = rows.copy()
    masked[1:, 3] = 0.0
    np.testing.assert_array_equal(alone, gpu_fid(job, masked, step_method="taylor", precision=1))
    assert np.any(both != alone)


def test_c2_subset_batches_consistently():
    """c2 (8 x 1H, blocks up to 70): 64 crystallites in one batch and in two."""
    cfg = W.config(2)
    rows = np.stack(cfg["powder"], axis=1)[:64]
    job = W.job_text(cfg)
    one = gpu_fid(job, rows)
    small = bl.Context(0, hbm_budget=6 << 30)  # ~160 MB per crystallite: forces two batches
    two = gpu_fid(job, rows, ctx=small)
    np.testing.assert_array_equal(one, two)


@pytest.mark.parametrize("seed,nsteps", [(0, 16), (1, 32), (2, 64), (3, 256), (6, 32), (10, 128)])
def test_twisted_fave_matches_oracle(seed, nsteps):
    """A power-of-two step count takes the twisted length-n correlation: all four rho/detect
    combinations of random_system (symmetric rho with and without mirrored block pairs,
    non-symmetric rho), against the oracle and against the direct correlation."""
    job, rows = random_system(seed)
    lines, kv = parse_job(job)
    job = job.replace(f"sw: {kv['sw']}", f"sw: {nsteps * float(kv['wr'])!r}")
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, fave_method="fft")
    assert rel(fid, ref) <= TOL, rel(fid, ref)
    assert rel(fid, gpu_fid(job, rows, fave_method="direct")) <= TOL


def quad2_system(seed):
    """A quadrupolar nucleus (spin 1 to 5/2) with one or two spin-1/2 partners, its Q line of
    order 0 (both terms), 1 (first order) or 2 (second order only) and a field chosen so the
    second-order coefficient Qp^2 / (B nu_rel) lands between 1 and 30 kHz."""
    rng = np.random.default_rng(1000 + seed)
    q = ["2H", "14N", "7Li", "23Na", "27Al", "17O"][seed % 6]
    rel_freq = {"2H": 61.424, "14N": 28.913, "7Li": 155.503, "23Na": 105.842, "27Al": 104.262,
                "17O": 54.242}[q] / 400.13
    others = [str(rng.choice(["1H", "13C"])) for _ in range(int(rng.integers(1, 3)))]
    iso = [q] + others
    n = len(iso)
    lines = [f"numspin {n}"] + [f"T {iso[k]} {k}" for k in range(n)]
    for k in range(n):
        a = rng.uniform(0, 360, 3)
        lines.append(f"C {rng.uniform(-2e3, 2e3):.9g} {rng.uniform(-6e3, 6e3):.9g} {rng.uniform(0, 1):.9g} {k} "
                     f"{a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    for i in range(n):
        for j in range(i + 1, n):
            a = rng.uniform(0, 360, 3)
            lines.append(f"D {rng.uniform(-1e4, 1e4):.9g} {i} {j} {a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    qp = float(rng.uniform(5e4, 4e5))
    order = seed % 3
    a = rng.uniform(0, 360, 3)
    lines.append(f"Q {qp:.9g} {rng.uniform(0, 1):.9g} 0 {a[0]:.9g} {a[1]:.9g} {a[2]:.9g} {order}")
    bfield = qp * qp / (rel_freq * float(rng.uniform(1e3, 3e4)))
    rho, det = [("Fx", "Fp"), ("Ix 0", "Ip 0"), ("Fx+Fz", "Fp")][seed % 3]
    wr = float(rng.uniform(8e3, 30e3)) if seed % 4 else 0.0
    n_steps = int(rng.integers(12, 50))
    job = "\n".join(f"spin: {l}" for l in lines) + (
        f"\nnpts: {int(rng.integers(50, 200))}\nsw: {(n_steps * wr if wr else 3e5)!r}\nwr: {wr!r}\n"
        f"rotb: {rng.uniform(30, 70)!r}\nrho: {rho}\ndet: {det}\nbfield: {bfield!r}\n")
    c = int(rng.integers(1, 24))
    rows = np.stack([rng.uniform(0, 2 * np.pi, c), np.arccos(rng.uniform(-1, 1, c)), rng.uniform(0, 2 * np.pi, c),
                     rng.uniform(0.1, 1, c)], axis=1)
    return job, rows


@pytest.mark.parametrize("method", ["eigh", "taylor"])
@pytest.mark.parametrize("seed", range(12))
def test_second_order_quadrupole_matches_oracle(seed, method):
    """SolidSys::setBfield: second-order quadrupolar terms for every Q order, quadrupolar
    spins 1 to 5/2, spinning and static, against the oracle."""
    job, rows = quad2_system(seed)
    ref, sw = oracle_fid(job, rows)
    fid, sw_g = gpu_fid(job, rows, return_sw=True, step_method=method)
    assert sw_g == sw
    assert rel(fid, ref) <= TOL, rel(fid, ref)


def test_tensor_core_blocks_of_41_and_50_mixed_within_1e6():
    """2H + 6 1H with a strong 2H-1H J (total Fz conserved): blocks 1,7,22,41,50,41,22,7,1.
    The mixed form runs the 41-blocks (up16 = 48: the stacked tiles' lower quarter has no rows)
    and the 50-block (up16 = 64) on the stacked tensor-core step and Dyson kernels; <= 1e-6
    against the oracle, and a crystallite alone equals it beside another bit for bit."""
    rng = np.random.default_rng(4141)
    lines = ["numspin 7", "T 2H 0"] + [f"T 1H {k}" for k in range(1, 7)]
    a = rng.uniform(0, 360, 3)
    lines.append(f"Q {rng.uniform(5e4, 1.5e5):.9g} {rng.uniform(0, 1):.9g} 0 {a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    for k in range(1, 7):
        a = rng.uniform(0, 360, 3)
        lines.append(f"C {rng.uniform(-2e3, 2e3):.9g} {rng.uniform(-6e3, 6e3):.9g} {rng.uniform(0, 1):.9g} {k} "
                     f"{a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    for i in range(7):
        for j in range(i + 1, 7):
            a = rng.uniform(0, 360, 3)
            lines.append(f"D {rng.uniform(-1.2e4, 1.2e4):.9g} {i} {j} {a[0]:.9g} {a[1]:.9g} {a[2]:.9g}")
    lines.append("J 60 0 1 1")
    assert sorted(bl.SolidSys(lines).blocks())[-3:] == [41, 41, 50]
    wr = 20e3
    job = "\n".join(f"spin: {l}" for l in lines) + (
        f"\nnpts: 300\nsw: {24 * wr!r}\nwr: {wr!r}\nrotb: {W.MAGIC_ANGLE!r}\nrho: Fx\ndet: Fp\n")
    rows = np.stack([rng.uniform(0, 2 * np.pi, 2), np.arccos(rng.uniform(-1, 1, 2)), rng.uniform(0, 2 * np.pi, 2),
                     rng.uniform(0.1, 1, 2)], axis=1)
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, step_method="taylor", precision=1)
    assert 0 < rel(fid, ref) <= 1e-6, rel(fid, ref)
    masked = rows.copy()
    masked[1, 3] = 0.0
    np.testing.assert_array_equal(gpu_fid(job, rows[:1], step_method="taylor", precision=1),
                                  gpu_fid(job, masked, step_method="taylor", precision=1))


def test_tensor_core_step_squarings_mixed_within_1e6():
    """c2's spin system at 10 steps per rotor period: the scaled step norm is ~4, so every
    tensor-core step (blocks 56 on the stacked kernel, 70 on the other) takes squarings;
    <= 1e-6 against the oracle."""
    cfg = W.config(2)
    cfg = dict(cfg, sw=10 * cfg["wr"], npts=200)
    job = W.job_text(cfg)
    rows = np.stack(cfg["powder"], axis=1)[:2]
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, step_method="taylor", precision=1)
    assert 0 < rel(fid, ref) <= 1e-6, rel(fid, ref)


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("precision", [0, 1])
def test_few_steps_per_period_match_oracle(n, precision):
    """1-3 steps per rotor period (the gamma loop sums 10, 5 and 3 shifted runs): Fave's
    transforms of length 2-8, below the three-stage register passes (the plain load and the
    one- and two-stage passes) in both forms."""
    job, rows = random_system(7)
    lines, kv = parse_job(job)
    job = job.replace(f"sw: {kv['sw']}", f"sw: {n * float(kv['wr'])!r}")
    ref, _ = oracle_fid(job, rows)
    fid = gpu_fid(job, rows, step_method="taylor", precision=precision)
    assert rel(fid, ref) <= (TOL if precision == 0 else 1e-6), rel(fid, ref)
