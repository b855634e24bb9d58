"""Seeded synthetic spin systems and powder sets for the five benchmark configurations.

No public dataset exists for this path: every input is generated here from a fixed seed
(0xB10C00 + config index; per system + system index) in the reference's own units (Hz
for couplings and shifts, degrees for Euler and rotor angles, radians in powder files).

  c0  13C-1H (dim 4): 13C CSA (iso U(-50,50) ppm, aniso U(20,150) ppm, eta U(0,1) at
      100 Hz/ppm, Euler U(0,360)), heteronuclear dipole b U(5,25) kHz with random PAS
      angles; rho = Ix(13C), detect = I+(13C); 10 kHz MAS, 100 steps, 1024 points,
      3-angle ZCW 1154.
  c1  4 x 1H (dim 16): coordinates U(0,4 A)^3, dipoles from r^-3 (120.07 kHz A^3),
      CSA aniso U(0,10) ppm at 400 Hz/ppm, eta U(0,1), iso 0, Euler U(0,360);
      rho = Fx, detect = F+; 20 kHz MAS, 128 steps, 2048 points, 3-angle ZCW 3722.
  c2  8 x 1H (dim 256): coordinates in a 5 A cube with 1.5 A minimum separation, all 28
      dipoles, CSA as c1; 30 kHz MAS, 200 steps, 4096 points, ZCW 1154.
  c3  512 systems of 2..7 1H (dims 4..128), dipoles + CSA as c2, weak J U(0,200) Hz,
      MAS U(5,35) kHz, U{64..256} steps, 1024 points, powders drawn from {144, 320, 678,
      1154}: the reference's repulsion sets crystals/rep144, rep320, rep678 (677 points,
      gamma = 0) and the 3-angle ZCW 1154.
  c4  the serving stream: c3-like jobs plus large jobs of 9..10 1H (dims 512..1024) drawn
      like c3 on the reference's 100-point repulsion set crystals/rep100 (config(4, i)).

Dipole sign: BlochLib's 'D del' enters H as del*(3cos^2-1)/2*(2IzSz - IxSx - IySy), so
the physical homonuclear coupling is del = -b with b = 120.07 kHz / r^3 (r in A).
"""
import math

import numpy as np

SEED0 = 0xB10C00
MAGIC_ANGLE = 54.7356
B_1H1H = 120.07e3  # Hz * A^3

# 3-angle ZCW lattices: alpha_j = 2pi frac(j a/N), beta_j = acos(2 frac(j b/N) - 1),
# gamma_j = 2pi frac(j g/N), w = 1/N.  (N, a, b, g) reproduce the reference's
# crystals/ZCW_3_1154 and ZCW_3_3722 files to ~1e-12.
ZCW3 = {1154: (271, 1, 107), 3722: (1483, 653, 1005)}


def zcw3(N, a=None, b=None, g=None):
    """(phi, theta, gamma, weight) arrays in the reference's powder-file column order."""
    if a is None:
        if N not in ZCW3:
            raise ValueError(f"no 3-angle ZCW generator stored for N={N}")
        a, b, g = ZCW3[N]
    j = np.arange(N, dtype=np.float64)
    frac = lambda x: x - np.floor(x)
    alpha = 2 * np.pi * frac(j * a / N)
    beta = np.arccos(2 * frac(j * b / N) - 1)
    gamma = 2 * np.pi * frac(j * g / N)
    w = np.full(N, 1.0 / N)
    return alpha, beta, gamma, w


_REP = None


def rep(N):
    """The reference's repulsion powder set crystals/rep<N> (N in 100, 144, 320, 678; rep678
    holds 677 points) as (phi, theta, gamma, weight); stored in data/rep_powders.npz by
    data/make_powders.py."""
    global _REP
    if _REP is None:
        from pathlib import Path
        with np.load(Path(__file__).resolve().parent / "data" / "rep_powders.npz") as z:
            _REP = {k: z[k] for k in z.files}
    a = _REP[f"rep{N}"]
    return tuple(np.array(a[i]) for i in range(4))


def _euler(rng):
    return rng.uniform(0, 360), math.degrees(math.acos(rng.uniform(-1, 1))), rng.uniform(0, 360)


def _proton_cluster(rng, nspin, box, min_sep=None):
    while True:
        xyz = rng.uniform(0, box, size=(nspin, 3))
        if min_sep is None:
            d = [np.linalg.norm(xyz[i] - xyz[j]) for i in range(nspin) for j in range(i + 1, nspin)]
            if min(d) > 1e-3:
                return xyz
            continue
        ok = all(np.linalg.norm(xyz[i] - xyz[j]) >= min_sep for i in range(nspin) for j in range(i + 1, nspin))
        if ok:
            return xyz


def _dipole_lines(xyz):
    lines = []
    n = len(xyz)
    for i in range(n):
        for j in range(i + 1, n):
            d = xyz[j] - xyz[i]
            r = float(np.linalg.norm(d))
            b = B_1H1H / r ** 3
            al = math.degrees(math.atan2(d[1], d[0]))
            be = math.degrees(math.acos(max(-1.0, min(1.0, d[2] / r))))
            lines.append(f"D {-b:.10g} {i} {j} {al:.10g} {be:.10g} 0")
    return lines


def _csa_lines(rng, nspin, hz_per_ppm=400.0, max_ppm=10.0):
    out = []
    for k in range(nspin):
        a, b, g = _euler(rng)
        out.append(f"C 0 {rng.uniform(0, max_ppm) * hz_per_ppm:.10g} {rng.uniform(0, 1):.10g} {k} "
                   f"{a:.10g} {b:.10g} {g:.10g}")
    return out


def config(index, system=0):
    """Workload dict: spin lines, rho/det expressions, params and powder arrays."""
    rng = np.random.default_rng(SEED0 + index + (system if index in (3, 4) else 0))
    if index == 0:
        a, b, g = rng.uniform(0, 360, 3)
        iso = rng.uniform(-50, 50) * 100.0
        dl = rng.uniform(20, 150) * 100.0
        eta = rng.uniform(0, 1)
        da, db, dg = _euler(rng)
        bd = rng.uniform(5, 25) * 1e3
        lines = ["numspin 2", "T 13C 0", "T 1H 1",
                 f"C {iso:.10g} {dl:.10g} {eta:.10g} 0 {a:.10g} {b:.10g} {g:.10g}",
                 f"D {bd:.10g} 0 1 {da:.10g} {db:.10g} {dg:.10g}"]
        return dict(name="c0", lines=lines, rho="Ix 0", det="Ip 0", npts=1024, wr=10e3, sw=100 * 10e3,
                    rotb=MAGIC_ANGLE, powder=zcw3(1154))
    if index == 1:
        xyz = _proton_cluster(rng, 4, 4.0)
        lines = ["numspin 4"] + [f"T 1H {k}" for k in range(4)] + _csa_lines(rng, 4) + _dipole_lines(xyz)
        return dict(name="c1", lines=lines, rho="Fx", det="Fp", npts=2048, wr=20e3, sw=128 * 20e3,
                    rotb=MAGIC_ANGLE, powder=zcw3(3722))
    if index == 2:
        xyz = _proton_cluster(rng, 8, 5.0, min_sep=1.5)
        lines = ["numspin 8"] + [f"T 1H {k}" for k in range(8)] + _csa_lines(rng, 8) + _dipole_lines(xyz)
        return dict(name="c2", lines=lines, rho="Fx", det="Fp", npts=4096, wr=30e3, sw=200 * 30e3,
                    rotb=MAGIC_ANGLE, powder=zcw3(1154))
    if index in (3, 4):
        nspin = int(rng.integers(2, 8)) if index == 3 else int(rng.integers(9, 11))
        xyz = _proton_cluster(rng, nspin, 5.0, min_sep=1.5)
        lines = ["numspin %d" % nspin] + [f"T 1H {k}" for k in range(nspin)] + _csa_lines(rng, nspin) + _dipole_lines(xyz)
        for i in range(nspin):
            for j in range(i + 1, nspin):
                lines.append(f"J {rng.uniform(0, 200):.10g} {i} {j}")
        wr = float(rng.uniform(5e3, 35e3))
        n = int(rng.integers(64, 257))
        if index == 3:
            npow = int(rng.choice([144, 320, 678, 1154]))
            pw = zcw3(1154) if npow == 1154 else rep(npow)
        else:
            pw = rep(100)
        return dict(name=f"c{index}.{system}", lines=lines, rho="Fx", det="Fp", npts=1024, wr=wr, sw=n * wr,
                    rotb=MAGIC_ANGLE, powder=pw)
    raise ValueError(index)


def subset(pw, count, start=0):
    """First `count` crystallites of a powder (phi, theta, gamma, weight) tuple."""
    return tuple(np.asarray(x)[start:start + count] for x in pw)


def job_text(cfg):
    """The job in the text format of oracle/ref_harness.cc (without the powder line)."""
    out = [f"spin: {l}" for l in cfg["lines"]]
    out += [f"npts: {cfg['npts']}", f"sw: {cfg['sw']!r}", f"wr: {cfg['wr']!r}", f"rotb: {cfg['rotb']!r}",
            f"rho: {cfg['rho']}", f"det: {cfg['det']}"]
    return "\n".join(out) + "\n"
