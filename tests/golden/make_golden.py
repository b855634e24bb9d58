#!/usr/bin/env python3
"""Generates the golden FID fixtures by running the BlochLib reference itself.

Run where the reference tree is present (BLOCHLIB_REF, resolved by oracle/build_ref.sh):
    oracle/build_ref.sh all && python3 tests/golden/make_golden.py
    (--hamgen, --writers, --p2p, ...: the other fixture sets, see main())

Each case is a seeded job in the text format of oracle/ref_harness.cc.  For every case
the fixture holds the job text, the crystallites (phi, theta, gamma, weight rows), the
FID of the reference built with its QL eigen-iteration in double (ref_fid64, the FP64
oracle) and as shipped (ref_fid, float QL), and the sweep width the reference reports.
Also recorded: the reference's built-in 2-angle ZCW sets, and sample rows of its
3-angle ZCW powder files (to check the closed-form generator in workloads.py).
"""
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from blochlib_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent
from blochlib_gb300.build import reference_tree  # noqa: E402

REF = reference_tree() or Path(os.environ.get("BLOCHLIB_REF", "reference-not-found"))
BIN64 = ROOT / "oracle" / "_ref" / "ref_fid64"
BIN32 = ROOT / "oracle" / "_ref" / "ref_fid"


def run_ref(binary, job_text, rows):
    with tempfile.TemporaryDirectory() as td:
        pw = Path(td) / "powder.txt"
        with open(pw, "w") as f:
            for r in rows:
                f.write(" ".join("%.17g" % x for x in r) + "\n")
        job = Path(td) / "job.txt"
        job.write_text(job_text + f"powder: {pw}\n")
        out = Path(td) / "out.bin"
        subprocess.run([str(binary), str(job), str(out)], check=True, timeout=1800)
        a = np.fromfile(out, dtype=np.float64)
    return float(a[0]), a[1:].view(np.complex128).copy()


def spread(n_total, k):
    return np.linspace(0, n_total - 1, k).round().astype(int)


def powder_rows(pw, idx):
    phi, theta, gamma, w = pw
    return np.stack([phi[idx], theta[idx], gamma[idx], w[idx]], axis=1)


def cases():
    c0 = W.config(0)
    yield "c0_sub16", W.job_text(c0), powder_rows(c0["powder"], spread(1154, 16))
    c1 = W.config(1)
    yield "c1_sub8", W.job_text(c1), powder_rows(c1["powder"], spread(3722, 8))
    c1n = dict(c1, rho="Fx+Fz", npts=512)
    yield "c1_nonsym_sub4", W.job_text(c1n), powder_rows(c1["powder"], spread(3722, 4))
    quad = dict(lines=["numspin 2", "T 2H 0", "T 13C 1", "Q 120000 0.3 0 10 20 30",
                       "C 500 4000 0.2 1 5 6 7", "D 2000 0 1 30 40 50", "J 50 0 1"],
                rho="Ix 0", det="Ip 0", npts=300, wr=5000.0, sw=200000.0, rotb=W.MAGIC_ANGLE)
    yield "quad_2h13c", W.job_text(quad), powder_rows(c0["powder"], spread(1154, 8))
    js = dict(lines=["numspin 3", "T 1H 0", "T 1H 1", "T 1H 2", "C 120 3000 0.4 0 10 20 30",
                     "C -80 2500 0.7 1 40 50 60", "C 0 1800 0.1 2 70 80 90", "D -15000 0 1 0 30 0",
                     "D -9000 1 2 50 60 0", "D -6000 0 2 120 100 0", "J 140 0 1 1", "J 70 1 2"],
              rho="Ix 0", det="Ix 0", npts=400, wr=15000.0, sw=96 * 15000.0, rotb=W.MAGIC_ANGLE)
    yield "jstrong_3h", W.job_text(js), powder_rows(c0["powder"], spread(1154, 6))
    gl = dict(lines=["numspin 2", "T 13C 0", "T 1H 1", "C 1500 6000 0.5 0 10 70 30", "D 8000 0 1 20 30 40"],
              rho="Ix 0", det="Ip 0", npts=64, wr=10000.0, sw=40000.0, rotb=W.MAGIC_ANGLE)
    yield "gammaloop_n4", W.job_text(gl), powder_rows(c0["powder"], spread(1154, 8))
    het = dict(lines=["numspin 3", "T 13C 0", "T 1H 1", "T 1H 2", "C 900 7000 0.6 0 33 44 55",
                      "D 9000 0 1 10 20 30", "D 7000 0 2 40 50 60", "D -20000 1 2 70 80 0"],
               rho="Ix 0", det="Ip 0", npts=512, wr=12000.0, sw=80 * 12000.0, rotb=30.0)
    yield "hetero_13c2h_30deg", W.job_text(het), powder_rows(c0["powder"], spread(1154, 6))
    st = dict(c0, npts=256)
    yield "c0_start_t", W.job_text(st) + "start: 1.7e-05\n", powder_rows(c0["powder"], spread(1154, 4))
    # static powder FIDs (oneFID.h:220-336): no spinning, and spinning with rotor angle 0
    s1 = dict(c1, wr=0.0, sw=200000.0, npts=512)
    yield "static_c1_wr0", W.job_text(s1), powder_rows(c1["powder"], spread(3722, 6))
    s0 = dict(c0, rotb=0.0, sw=250000.0, npts=400)
    yield "static_c0_rotb0", W.job_text(s0), powder_rows(c0["powder"], spread(1154, 8))
    sq = dict(quad, wr=0.0, rotb=35.0, sw=500000.0, npts=256)
    yield "static_quad_tilted", W.job_text(sq), powder_rows(c0["powder"], spread(1154, 5))
    sn = dict(js, wr=0.0, rho="Fx+Fz", det="Fp", sw=300000.0, npts=300)
    yield "static_jstrong_nonsym", W.job_text(sn), powder_rows(c0["powder"], spread(1154, 5))


def big_cases():
    """Systems with Hamiltonian blocks larger than 8 (5, 6 and 8 like spins)."""
    c0 = W.config(0)
    c3 = W.config(3, 1)  # a seeded c3 system
    for nspin, seed, name in [(5, 11, "big_5h"), (6, 12, "big_6h")]:
        rng = np.random.default_rng(W.SEED0 + seed)
        xyz = W._proton_cluster(rng, nspin, 5.0, min_sep=1.5)
        lines = [f"numspin {nspin}"] + [f"T 1H {k}" for k in range(nspin)] + W._csa_lines(rng, nspin) + \
            W._dipole_lines(xyz) + ["J 85 0 1"]
        cfg = dict(lines=lines, rho="Fx", det="Fp", npts=512, wr=25000.0, sw=50 * 25000.0, rotb=W.MAGIC_ANGLE)
        yield name, W.job_text(cfg), powder_rows(c0["powder"], spread(1154, 3 if nspin == 5 else 2))
    c2 = W.config(2)
    yield "c2_sub1", W.job_text(c2), powder_rows(c2["powder"], spread(1154, 1))


def huge_cases():
    """9 like spins (dim 512; blocks 1,9,36,84,126,126,84,36,9,1): blocks above 74 take the
    batched-product path; one crystallite, few steps, so that the dense reference is quick."""
    c0 = W.config(0)
    for seed, name, rho, nstep in [(21, "huge_9h", "Fx", 12), (22, "huge_9h_nonsym", "Fx+Fz", 10)]:
        rng = np.random.default_rng(W.SEED0 + seed)
        xyz = W._proton_cluster(rng, 9, 6.0, min_sep=1.5)
        lines = ["numspin 9"] + [f"T 1H {k}" for k in range(9)] + W._csa_lines(rng, 9) + W._dipole_lines(xyz) + \
            ["J 75 0 1", "J 40 3 4"]
        cfg = dict(lines=lines, rho=rho, det="Fp", npts=96, wr=25000.0, sw=nstep * 25000.0, rotb=W.MAGIC_ANGLE)
        yield name, W.job_text(cfg), powder_rows(c0["powder"], spread(1154, 1) + 300)


def quad2_cases():
    """Second-order quadrupolar terms (SolidSys::setBfield): 2H with two 1H (both orders),
    27Al with 1H (Q line order 2: second order only), and a static case.  The fields are small
    so that the second-order term is large against the FP64 parity bar."""
    c0 = W.config(0)
    base = ["T 2H 0", "T 1H 1", "T 1H 2", "C 300 2500 0.4 1 10 40 70", "D -9000 1 2 20 50 0",
            "D 3000 0 1 60 80 0", "D 2000 0 2 100 30 0"]
    mas = dict(npts=256, wr=20000.0, sw=40 * 20000.0, rotb=W.MAGIC_ANGLE, rho="Fx", det="Fp")
    cfg = dict(mas, lines=["numspin 3"] + base + ["Q 160000 0.3 0 30 60 90"])
    yield "quad2_2h1h", W.job_text(cfg) + "bfield: 200000\n", powder_rows(c0["powder"], spread(1154, 5))
    al = ["numspin 2", "T 27Al 0", "T 1H 1", "C 800 1500 0.2 1 0 30 0", "D 4000 0 1 20 70 0",
          "Q 2500000 0.5 0 15 45 75 2"]
    cfg = dict(mas, lines=al, rho="Ix 0", det="Ip 0", wr=25000.0, sw=32 * 25000.0)
    yield "quad2_only_27al", W.job_text(cfg) + "bfield: 5000000\n", powder_rows(c0["powder"], spread(1154, 4))
    cfg = dict(mas, lines=["numspin 3"] + base + ["Q 160000 0.3 0 30 60 90"], wr=0.0, sw=400000.0, npts=200)
    yield "static_quad2", W.job_text(cfg) + "bfield: 200000\n", powder_rows(c0["powder"], spread(1154, 4))
    # 2H with n protons: n = 4 (dim 48, largest Fz block 14: per-crystallite CTA path) and
    # n = 7 (dim 384, largest block 91: batched-product path; kept out of the dense oracle)
    for n, name, nstep, ncry in [(4, "quad2_big_2h4h", 24, 3), (7, "huge_quad2_2h7h", 10, 1)]:
        rng = np.random.default_rng(W.SEED0 + 40 + n)
        xyz = W._proton_cluster(rng, n + 1, 5.0, min_sep=1.5)
        dips = [l for l in W._dipole_lines(xyz)]
        lines = [f"numspin {n + 1}", "T 2H 0"] + [f"T 1H {k}" for k in range(1, n + 1)] + \
            W._csa_lines(rng, n + 1)[1:] + dips + ["Q 140000 0.6 0 20 70 10"]
        cfg = dict(lines=lines, rho="Fx", det="Fp", npts=96, wr=25000.0, sw=nstep * 25000.0, rotb=W.MAGIC_ANGLE)
        yield name, W.job_text(cfg) + "bfield: 250000\n", powder_rows(c0["powder"], (spread(1154, ncry) + 200) % 1154)


def p2p_cases():
    """Point-to-point FIDs (ref_harness 'p2p: base factor'): dwell = factor/base rotor periods,
    chunks of ceil(chunk/maxtstep) steps.  base < factor runs the reference's own
    PropReduce::reduce + generateProps; the others form the same dwell products directly."""
    c0, c1 = W.config(0), W.config(1)
    het = ["numspin 3", "T 13C 0", "T 1H 1", "T 1H 2", "C 900 7000 0.6 0 33 44 55", "D 9000 0 1 10 20 30",
           "D 7000 0 2 40 50 60", "D -20000 1 2 70 80 0"]
    js = ["numspin 3", "T 1H 0", "T 1H 1", "T 1H 2", "C 120 3000 0.4 0 10 20 30", "C -80 2500 0.7 1 40 50 60",
          "C 0 1800 0.1 2 70 80 90", "D -15000 0 1 0 30 0", "D -9000 1 2 50 60 0", "D -6000 0 2 120 100 0",
          "J 140 0 1 1", "J 70 1 2"]
    q2 = ["numspin 2", "T 2H 0", "T 1H 1", "C 300 2500 0.4 1 10 40 70", "D 3000 0 1 60 80 0",
          "Q 160000 0.3 0 30 60 90"]
    mas = dict(rotb=W.MAGIC_ANGLE, sw=0.0)
    cases = [
        ("p2p_het_9_7", dict(mas, lines=het, rho="Ix 0", det="Ip 0", npts=160, wr=10000.0), "9 7", 3e-6, 6, ""),
        ("p2p_jstrong_7_9_nonsym", dict(mas, lines=js, rho="Fx+Fz", det="Fp", npts=128, wr=15000.0), "7 9", 2e-6,
         5, ""),
        ("p2p_quad2_5_3", dict(mas, lines=q2, rho="Fx", det="Fp", npts=128, wr=20000.0), "5 3", 2e-6, 5,
         "bfield: 200000\n"),
        ("p2p_c1_sync_1_1", dict(c1, npts=96), "1 1", 5e-6, 4, ""),
        ("p2p_het_2_3_start", dict(mas, lines=het, rho="Ix 0", det="Ip 0", npts=100, wr=12000.0), "2 3", 0.0, 4,
         "start: 1.3e-05\n"),
        ("p2p_static", dict(lines=het, rho="Ix 0", det="Ip 0", npts=128, wr=0.0, sw=100000.0,
                            rotb=W.MAGIC_ANGLE), "1 1", 0.0, 6, ""),
    ]
    for name, cfg, bf, mt, ncry, extra in cases:
        yield name, W.job_text(cfg) + f"p2p: {bf}\nmaxtstep: {mt!r}\n" + extra, \
            powder_rows(c0["powder"], (spread(1154, ncry) + 77) % 1154)
    # large blocks (5 like spins, blocks up to 10): base 4, factor 1
    rng = np.random.default_rng(W.SEED0 + 11)
    xyz = W._proton_cluster(rng, 5, 5.0, min_sep=1.5)
    lines = ["numspin 5"] + [f"T 1H {k}" for k in range(5)] + W._csa_lines(rng, 5) + W._dipole_lines(xyz)
    cfg = dict(lines=lines, rho="Fx", det="Fp", npts=64, wr=25000.0, sw=0.0, rotb=W.MAGIC_ANGLE)
    yield "p2p_big_5h_4_1", W.job_text(cfg) + "p2p: 4 1\nmaxtstep: 2e-06\n", powder_rows(c0["powder"], spread(1154, 2))


HAMGEN_SYSTEMS = {
    "h_c_d": ["numspin 3", "T 1H 0", "T 13C 1", "T 2H 2"],
    "hh": ["numspin 2", "T 1H 0", "T 1H 1"],
}
HAMGEN_EXPRS = [
    # spin operators: totals, single spins, every Cartesian name
    "Ix", "Iy", "Iz", "Ip", "Im", "Ie", "Ix_0", "Iy_1", "Iz_2", "Ip_2", "Im_1", "Ie_2",
    # arithmetic, variables, precedence
    "Ix_0 + Iz_1", "Ix_0 - Iz_1", "2*Ix_0", "Ix_0*2", "Ix_0/2", "2/Iz_0", "Ix_0/Iz_0", "complexi*Iy_1",
    "Ix_0 + complexi*Iy_0", "pi*Iz_1", "deg2rad*90*Ix_2", "e*Ie_0", "Pi*PI/pi*rad2deg*Iz_0", "Iz_0*Iz_1",
    "Ip_0*Im_1 + Im_0*Ip_1", "(Ix_0+Iy_1)*(Ix_0-Iy_1)", "((Ix_0+Iz_1)*2 - Iy_2)/3", "-Ix_0", "+Ix_1",
    "Ix_0 + 1", "1 - Iz_0", "Iz_0 - 1", "1 + 2 + Iz_0", "6/2*Iz_0", "2*3*4*Iz_0", "1.5e1*Iz_0", "2e-1*Iz_0",
    ".5*Iz_0", "2.5E0*Iz_0",
    # quirks of the reference's parser and evaluator
    "Iz_1^2", "Ix_2^3", "Iz_0^0", "Iz_0^-1", "Iz_0^2.7", "-2^2*Iz_0", "2*-3*Iz_0", "2^3^2*Iz_0",
    "Ix_0 Iz_1", "Ixy", "Ix_0 = Iz_0", "Ix_0 & Iz_0", "frac(2)*Iz_0", "round(2.5)*Iz_0", "trunc(3.3)*Iz_0",
    # spin tensors
    "T00_1", "T10_0", "T11_0", "T1m1_2", "T20_0,1", "T21_0,2", "T2m1_1,2", "T22_2", "T2m2_0,2", "T20_2",
    # spatial tensors of the powder angles
    "A20*Iz_0", "A21*T2m1_0,1 + A2m1*T21_0,1", "A10*Iz_1", "A11*Ix_0", "A1m1*Iy_0", "A22*T2m2_0,1",
    "A2m2*T22_0,1", "A00*Ix_0",
    # functions on matrices (element by element)
    "exp(Iz_0)", "sqrt(Iz_0)", "abs(Iy_0)", "real(Iy_0)", "imag(Iy_0)", "ceil(Iz_0)", "floor(Iz_0)",
    "cos(Ix_0)", "sin(Ix_0)", "tan(Iz_0)", "sinh(Iz_0)", "cosh(Iz_0)", "tanh(Iz_0)", "ln(Ix_0+2)",
    "log(Ix_0+2)", "acos(Iz_0)", "asin(Iz_0)", "atan(Iz_0)", "-(Ix_0)", "exp(complexi*Iz_0)",
    # functions and logic on numbers
    "sqrt(2)*Iz_0", "exp(1)*Ix_0", "ln(2)*Iz_0", "log(100)*Iz_0", "cos(pi/3)*Ix_0", "sin(pi/6)*Iy_0",
    "tan(1)*Iz_0", "acos(0.5)*Iz_0", "asin(0.5)*Iz_0", "atan(1)*Iz_0", "sinh(1)*Iz_0", "cosh(1)*Iz_0",
    "tanh(0.5)*Iz_0", "abs(-3)*Iz_0", "int(2.7)*Iz_0", "ceil(2.1)*Iz_0", "floor(2.9)*Iz_0", "2^3*Iz_0",
    "(2>1)*Iz_0", "(1>2)*Iz_0 + Ix_0", "(2<=2)*Iz_0", "(3>=4)*Iz_0 + Ix_0", "(3==3)*Iz_0",
    "(3!=3)*Iz_0 + Ix_0", "(1&&0)*Iz_0 + Ix_0", "(1||0)*Iz_0", "(7%3)*Iz_0", "!0*Iz_0", "(-3>2)*Iz_0",
    "real(complexi)*Iz_0 + Ix_0", "imag(complexi)*Iz_0", "sqrt(-4)*Iz_0", "ln(-1)*Iz_0", "log(complexi)*Iz_0",
    "(2+complexi)^(1-complexi)*Iz_0", "acos(2)*Iz_0", "atan(complexi/2)*Iz_0",
    # user variables (added with addVar)
    "w1*Ix_0 + w2*Iy_0",
]
HAMGEN_VARS = {"w1": complex(2.5, 0.0), "w2": complex(0.0, -1.25)}
HAMGEN_ANGLES = [(0.7, 1.1, 0.3), (2.0, -0.4, 0.0)]


def hamgen_fixtures():
    """Matrices of the reference's HamiltonianGen (ref_harness 'hamgen:'), one process per
    expression (a reference exception then loses only that expression).  User variables are
    substituted textually for the reference, which has no job key for them."""
    out = {}
    for sname, lines in HAMGEN_SYSTEMS.items():
        for ai, ang in enumerate(HAMGEN_ANGLES):
            for ei, ex in enumerate(HAMGEN_EXPRS):
                if sname == "hh" and any(t in ex for t in ("_2", "T22_2", "T20_2")):
                    continue
                rex = ex
                for k, v in HAMGEN_VARS.items():  # no "*-": the reference drops that sign
                    rex = rex.replace(k, f"({v.real!r}{'+' if v.imag >= 0 else '-'}complexi*{abs(v.imag)!r})")
                job = "".join(f"spin: {l}\n" for l in lines) + f"hamgen_angles: {ang[0]!r} {ang[1]!r} {ang[2]!r}\n"
                job += f"hamgen: {rex}\n"
                with tempfile.TemporaryDirectory() as td:
                    (Path(td) / "j.txt").write_text(job)
                    r = subprocess.run([str(BIN64), str(Path(td) / "j.txt"), str(Path(td) / "o.bin")],
                                       capture_output=True, timeout=60)
                    if r.returncode != 0:
                        print("reference failed:", sname, ex, r.stderr.decode()[-200:])
                        continue
                    a = np.fromfile(Path(td) / "o.bin")
                n = int(a[0])
                out[f"{sname}|{ai}|{ei}"] = a[1:1 + 2 * n * n].view(np.complex128).reshape(n, n)
    np.savez_compressed(OUT / "hamgen.npz", **out,
                        _exprs=np.array(HAMGEN_EXPRS), _angles=np.array(HAMGEN_ANGLES),
                        _systems=np.array(json.dumps(HAMGEN_SYSTEMS)), _vars=np.array(json.dumps(
                            {k: [v.real, v.imag] for k, v in HAMGEN_VARS.items()})))
    print("hamgen fixtures:", len(out))


def rf_cases():
    """Continuous rf during the FID (ref_harness 'rf:': SolidSys wrapped in a Func_T that adds
    solid-2.0's PulseData::Pulse term), for oneFID::FID (spinning and static) and the
    point-to-point form."""
    c0 = W.config(0)
    ch = ["numspin 2", "T 13C 0", "T 1H 1", "C 1500 6000 0.5 0 10 70 30", "D 8000 0 1 20 30 40"]
    het3 = ["numspin 3", "T 13C 0", "T 1H 1", "T 1H 2", "C 900 7000 0.6 0 33 44 55", "D 9000 0 1 10 20 30",
            "D 7000 0 2 40 50 60", "D -20000 1 2 70 80 0", "J 100 1 2 1"]
    q2 = ["numspin 2", "T 2H 0", "T 1H 1", "C 300 2500 0.4 1 10 40 70", "D 3000 0 1 60 80 0",
          "Q 160000 0.3 0 30 60 90"]
    mas = dict(rotb=W.MAGIC_ANGLE)
    cases = [
        ("rf_decouple_x", dict(mas, lines=ch, rho="Ix 0", det="Ip 0", npts=256, wr=10000.0, sw=400000.0),
         "rf: 1H 80000 0 0\n", 6),
        ("rf_decouple_y_offset", dict(mas, lines=ch, rho="Ix 0", det="Ip 0", npts=256, wr=10000.0, sw=400000.0),
         "rf: 1H 60000 90 2000\n", 6),
        ("rf_het3_30deg_strongj", dict(mas, lines=het3, rho="Fx", det="Fp", npts=256, wr=12000.0, sw=12000.0 * 32),
         "rf: 1H 50000 30 0\n", 5),
        ("rf_lock_13c_two_fields", dict(mas, lines=ch, rho="Ix 0", det="Ip 0", npts=256, wr=10000.0, sw=400000.0),
         "rf: 13C 20000 0 500\nrf: 13C 15000 90 0\nrf: 1H 0 45 3000\n", 6),
        ("static_rf_120deg", dict(mas, lines=ch, rho="Ix 0", det="Ip 0", npts=200, wr=0.0, sw=200000.0),
         "rf: 1H 70000 120 0\n", 6),
        ("p2p_rf_5_3", dict(mas, lines=het3, rho="Fx", det="Fp", npts=100, wr=12000.0, sw=0.0),
         "rf: 1H 50000 60 1000\np2p: 5 3\nmaxtstep: 3e-06\n", 4),
        ("rf_quad2_45deg", dict(mas, lines=q2, rho="Fx", det="Fp", npts=256, wr=20000.0, sw=20000.0 * 40),
         "rf: 2H 30000 45 0\nbfield: 200000\n", 5),
    ]
    for name, cfg, extra, ncry in cases:
        yield name, W.job_text(cfg) + extra, powder_rows(c0["powder"], (spread(1154, ncry) + 33) % 1154)
    # rf on like spins joins every Fz sector: 5 1H (one block of 32, the CTA kernels) and
    # 7 1H (one block of 128, the batched products)
    for n, name, nstep, ncry in [(5, "rf_lock_5h_big", 24, 2), (7, "huge_rf_lock_7h", 8, 1)]:
        rng = np.random.default_rng(W.SEED0 + 60 + n)
        xyz = W._proton_cluster(rng, n, 5.0, min_sep=1.5)
        lines = [f"numspin {n}"] + [f"T 1H {k}" for k in range(n)] + W._csa_lines(rng, n) + W._dipole_lines(xyz)
        cfg = dict(lines=lines, rho="Fx", det="Fp", npts=96, wr=25000.0, sw=nstep * 25000.0, rotb=W.MAGIC_ANGLE)
        yield name, W.job_text(cfg) + "rf: 1H 40000 0 0\n", powder_rows(c0["powder"], (spread(1154, ncry) + 500) % 1154)


def rfc_cases():
    """rf that changes within the rotor period, point-to-point form (ref_harness 'rfc:': one
    pulse term per chunk, on top of the continuous fields; base and factor as given)."""
    c0 = W.config(0)
    het3 = ["numspin 3", "T 13C 0", "T 1H 1", "T 1H 2", "C 900 7000 0.6 0 33 44 55", "D 9000 0 1 10 20 30",
            "D 7000 0 2 40 50 60", "D -20000 1 2 70 80 0"]
    q2 = ["numspin 2", "T 2H 0", "T 1H 1", "C 300 2500 0.4 1 10 40 70", "D 3000 0 1 60 80 0",
          "Q 160000 0.3 0 30 60 90"]
    base = dict(lines=het3, rho="Ix 0", det="Ip 0", npts=128, wr=10000.0, sw=0.0, rotb=W.MAGIC_ANGLE)
    cases = [
        ("p2p_rfc_window_9_7", base, "p2p: 9 7\nmaxtstep: 3e-06\n" + "".join(f"rfc: {k} 1H 80000 0 0\n" for k in range(5))),
        ("p2p_rfc_phase_cycle_4_1", base, "p2p: 4 1\nmaxtstep: 5e-06\n" + "".join(f"rfc: {k} 1H 50000 {90 * k} 0\n" for k in range(4))),
        ("p2p_rfc_cw13c_45deg_5_3", base, "p2p: 5 3\nmaxtstep: 4e-06\nrf: 13C 20000 0 300\n"
                                           "rfc: 1 1H 60000 45 1000\nrfc: 3 1H 60000 225 1000\n"),
        ("p2p_rfc_noncoprime_6_4", base, "p2p: 6 4\nmaxtstep: 4e-06\nrfc: 1 1H 70000 30 0\nrfc: 4 1H 70000 30 0\n"),
        ("p2p_rfc_quad2_4_3", dict(base, lines=q2, rho="Fx", det="Fp", wr=20000.0),
         "p2p: 4 3\nmaxtstep: 2e-06\nbfield: 200000\nrfc: 0 2H 40000 60 0\nrfc: 2 2H 40000 -60 0\n"),
    ]
    for name, cfg, extra in cases:
        yield name, W.job_text(cfg) + extra, powder_rows(c0["powder"], (spread(1154, 5) + 71) % 1154)
    rng = np.random.default_rng(W.SEED0 + 77)
    xyz = W._proton_cluster(rng, 5, 5.0, min_sep=1.5)
    lines = ["numspin 5"] + [f"T 1H {k}" for k in range(5)] + W._csa_lines(rng, 5) + W._dipole_lines(xyz)
    cfg = dict(lines=lines, rho="Fx", det="Fp", npts=64, wr=25000.0, sw=0.0, rotb=W.MAGIC_ANGLE)
    yield ("p2p_rfc_big_5h_3_2", W.job_text(cfg) + "p2p: 3 2\nmaxtstep: 3e-06\nrfc: 0 1H 50000 0 0\nrfc: 2 1H 50000 90 0\n",
           powder_rows(c0["powder"], spread(1154, 2)))


# FIDs written by the reference's own plotterFID (ref_harness 'writers:'): lengths that are
# and are not powers of two, sweep widths with long decimal expansions, values over 6 decades
WRITER_CASES = ((100, 1e-5, 1), (128, 2.5e-6, 2), (1000, 3.3e-5, 3), (4096, 1.6666666666666667e-07, 4),
                (7, 0.001, 5))


def writer_fixtures():
    """plotter_ref.npz: per case the FID, dt and the reference's plotterFID text, byte for byte."""
    out = {}
    for n, dt, seed in WRITER_CASES:
        rng = np.random.default_rng(seed)
        fid = rng.normal(size=n) * 10 ** rng.uniform(-3, 3) + 1j * rng.normal(size=n)
        with tempfile.TemporaryDirectory() as td:
            t = Path(td)
            np.ascontiguousarray(np.stack([fid.real, fid.imag], 1)).tofile(t / "fid.bin")
            (t / "j.txt").write_text(f"writers: {t / 'fid.bin'} {n} {dt!r} {t / 'fid.txt'} {t / 'fid.mat'}\n")
            r = subprocess.run([str(BIN64), str(t / "j.txt"), str(t / "unused.bin")], capture_output=True, timeout=60)
            if r.returncode != 0:
                sys.exit("reference writers failed: " + r.stderr.decode()[-300:])
            text = (t / "fid.txt").read_bytes()
        out[f"fid_{n}"] = fid
        out[f"dt_{n}"] = np.array(dt)
        out[f"text_{n}"] = np.frombuffer(text, dtype=np.uint8)
    np.savez_compressed(OUT / "plotter_ref.npz", **out)
    print("plotter fixtures:", len(WRITER_CASES))


def main():
    if "--hamgen" in sys.argv:
        hamgen_fixtures()
        return
    if "--writers" in sys.argv:
        writer_fixtures()
        return
    if not BIN64.exists():
        sys.exit("oracle/_ref/ref_fid64 missing: run oracle/build_ref.sh first")
    if any(a in sys.argv for a in ("--big", "--huge", "--quad2", "--p2p", "--rf", "--rfc")):
        man = json.loads((OUT / "manifest.json").read_text())
        extra = (huge_cases() if "--huge" in sys.argv else quad2_cases() if "--quad2" in sys.argv
                 else p2p_cases() if "--p2p" in sys.argv else rf_cases() if "--rf" in sys.argv
                 else rfc_cases() if "--rfc" in sys.argv else big_cases())
        for name, job, rows in extra:
            sw64, f64 = run_ref(BIN64, job, rows)
            np.savez_compressed(OUT / f"{name}.npz", job=np.array(job), powder=rows, fid64=f64, fid32=f64 * 0,
                                sw=np.array(sw64))
            man[name] = {"crystallites": len(rows), "npts": len(f64), "sw": sw64, "float_ql_rel_dev": None}
            print(name, man[name], flush=True)
        (OUT / "manifest.json").write_text(json.dumps(man, indent=1))
        return
    manifest = {}
    for name, job, rows in cases():
        sw64, f64 = run_ref(BIN64, job, rows)
        sw32, f32 = run_ref(BIN32, job, rows)
        np.savez_compressed(OUT / f"{name}.npz", job=np.array(job), powder=rows, fid64=f64, fid32=f32,
                            sw=np.array(sw64))
        manifest[name] = {"crystallites": len(rows), "npts": len(f64), "sw": sw64,
                          "float_ql_rel_dev": float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64))}
        print(name, manifest[name])
    # built-in 2-angle ZCW sets (powder.cc:248-280)
    zcw = {}
    for t, p in [(144, 89), (233, 144), (21, 8)]:
        with tempfile.TemporaryDirectory() as td:
            dump = Path(td) / "pw.bin"
            job = "spin: numspin 1\nspin: T 1H 0\nnpts: 1\nsw: 1000\nwr: 100\nrotb: 54.7356\nrho: Fx\ndet: Fp\n"
            jf = Path(td) / "job.txt"
            jf.write_text(job + f"powder_zcw: {t} {p}\ndump_powder: {dump}\n")
            subprocess.run([str(BIN64), str(jf), str(Path(td) / "o.bin")], check=True)
            zcw[f"{t}_{p}"] = np.fromfile(dump).reshape(-1, 4)
    np.savez_compressed(OUT / "zcw_builtin.npz", **zcw)
    # sample rows of the 3-angle ZCW powder files shipped with the reference
    samples = {}
    for n in (1154, 3722):
        rows = np.loadtxt(REF / "crystals" / f"ZCW_3_{n}")
        idx = [0, 1, 2, 3, 100, n // 2, n - 2, n - 1]
        samples[str(n)] = {"index": idx, "rows": rows[idx].tolist(), "count": int(len(rows))}
    (OUT / "zcw3_samples.json").write_text(json.dumps(samples, indent=1))
    (OUT / "manifest.json").write_text(json.dumps(manifest, indent=1))


if __name__ == "__main__":
    main()
