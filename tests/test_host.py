"""Host side of the boundary through the C ABI: spin systems, operators, blocks, powders,
FID text output and error statuses.  No GPU needed."""
import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W
from helpers import GOLDEN


def single(spin, which):
    hs = int(round(2 * spin + 1))
    q = (hs - 1) / 2
    m = np.zeros((hs, hs), dtype=complex)
    if which == "z":
        return np.diag(q - np.arange(hs)).astype(complex)
    for k in range(hs - 1):
        mm = q - 1 - k
        c = np.sqrt(q * (q + 1) - mm * (mm + 1))
        if which == "p":
            m[k, k + 1] = c
        elif which == "m":
            m[k + 1, k] = c
        elif which == "x":
            m[k, k + 1] = m[k + 1, k] = c / 2
        elif which == "y":
            m[k + 1, k], m[k, k + 1] = 0.5j * c, -0.5j * c
    return m


def expand(spins, k, op):
    out = np.eye(1, dtype=complex)
    for i, s in enumerate(spins):
        out = np.kron(out, op if i == k else np.eye(int(round(2 * s + 1))))
    return out


def test_operators_match_kronecker_construction():
    sys_ = bl.SolidSys(["numspin 3", "T 1H 0", "T 2H 1", "T 13C 2"])
    spins = [0.5, 1.0, 0.5]
    assert sys_.dim() == 12 and sys_.spins() == 3
    for k in range(3):
        for w, name in [("x", "Ix"), ("y", "Iy"), ("z", "Iz"), ("p", "Ip"), ("m", "Im")]:
            np.testing.assert_array_equal(sys_.op(f"{name} {k}"), expand(spins, k, single(spins[k], w)))
    tot = sum(expand(spins, k, single(spins[k], "p")) for k in range(3))
    np.testing.assert_array_equal(sys_.Fp(), tot)
    np.testing.assert_array_equal(sys_.op("0.5*Fx + Iz 1"),
                                  0.5 * sum(expand(spins, k, single(spins[k], "x")) for k in range(3))
                                  + expand(spins, 1, single(1.0, "z")))


def test_block_structure_follows_magnetisation_sectors():
    c1 = W.config(1)
    assert sorted(bl.SolidSys(c1["lines"]).blocks()) == [1, 1, 4, 4, 6]
    c0 = W.config(0)  # heteronuclear, secular: H is diagonal
    assert bl.SolidSys(c0["lines"]).blocks() == [1, 1, 1, 1]
    c2 = W.config(2)
    assert sorted(bl.SolidSys(c2["lines"]).blocks()) == [1, 1, 8, 8, 28, 28, 56, 56, 70]


def test_zcw_builtin_matches_reference():
    ref = np.load(GOLDEN / "zcw_builtin.npz")
    for key in ref.files:
        t, p = map(int, key.split("_"))
        th, ph, ga, w = bl.powder(bl.powder.zcw, t, p).arrays()
        r = ref[key]
        np.testing.assert_allclose(th, r[:, 0], rtol=0, atol=1e-15)
        np.testing.assert_allclose(ph, r[:, 1], rtol=0, atol=1e-15)
        np.testing.assert_array_equal(ga, r[:, 2])
        np.testing.assert_allclose(w, r[:, 3], rtol=1e-14, atol=0)


def test_powder_file_reader_column_rules(tmp_path):
    f = tmp_path / "p.txt"
    f.write_text("# comment\n% other comment\n0.1 0.2 0.3 0.4\n0.5 0.6 0.7\n0.8 0.9\n1.1\n")
    th, ph, ga, w = bl.powder.read(f).arrays()
    np.testing.assert_array_equal(ph, [0.1, 0.5, 0.8, 1.1])   # column 0 -> phi
    np.testing.assert_array_equal(th, [0.2, 0.6, 0.9, 0.0])   # column 1 -> theta
    np.testing.assert_array_equal(ga, [0.3, 0.0, 0.0, 0.0])   # 4 columns: gamma then weight
    np.testing.assert_array_equal(w, [0.4, 0.7, 1.0, 1.0])    # 3 columns: weight; fewer: 1


def test_plotter_fid_text_matches_the_reference_byte_for_byte(tmp_path):
    """plotterFID's 7-column text equals, byte for byte, what the reference's own plotterFID
    (utils/plotter.cc:49-135, run by tests/golden/make_golden.py --writers) wrote for the same
    FID and dt: lengths that are and are not powers of two (the reference's zero-fill drops the
    last point), values over six decades."""
    g = np.load(GOLDEN / "plotter_ref.npz")
    ns = sorted(int(k[4:]) for k in g.files if k.startswith("fid_"))
    assert len(ns) >= 5
    for n in ns:
        path = tmp_path / f"fid{n}.txt"
        bl.plotterFID(g[f"fid_{n}"], path, float(g[f"dt_{n}"]))
        assert path.read_bytes() == g[f"text_{n}"].tobytes(), n


def test_plotter_fid_text(tmp_path):
    rng = np.random.default_rng(1)
    fid = rng.normal(size=100) + 1j * rng.normal(size=100)
    path = tmp_path / "fid.txt"
    bl.plotterFID(fid, path, 1e-5)
    d = np.loadtxt(path)
    n = 128  # zero-filled to the next power of two
    assert d.shape == (n, 7)
    x = np.concatenate([fid, np.zeros(n - 100)])
    x[99] = 0  # the reference's zero-fill (resizeAndPreserve) overwrites the last point
    S = np.fft.ifft(x) * n  # the reference's FFT has the +i sign and no scaling
    S = np.roll(S, -(n // 2))
    np.testing.assert_allclose(d[:, 0], np.arange(n) * 1e-5, rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(d[:, 1], -0.5 / 1e-5 + np.arange(n) / (1e-5 * n), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(d[:, 2] + 1j * d[:, 3], S, rtol=2e-5, atol=1e-4)
    np.testing.assert_allclose(d[:, 4] + 1j * d[:, 5], x, rtol=2e-5, atol=1e-5)
    np.testing.assert_allclose(d[:, 6], np.abs(S), rtol=2e-5, atol=1e-4)


@pytest.mark.parametrize("lines,status", [
    (["numspin 2", "T 1H 0", "T 1H 5"], 2),
    (["numspin 2", "T 1H 0", "T Xx9 1"], 2),
    (["numspin 2", "C 1 2 0.1"], 2),
    (["numspin 2", "D 100 0 7"], 2),
    (["numspin 1", "T 1H 0", "Q 1000 0 0"], 2),
])
def test_malformed_systems_return_parse_status(lines, status):
    with pytest.raises(bl.BlochError) as e:
        bl.SolidSys(lines)
    assert e.value.status == status


def test_bad_zcw_and_operator_return_invalid():
    with pytest.raises(bl.BlochError) as e:
        bl.powder(bl.powder.zcw, 100, 7)
    assert e.value.status == 1
    s = bl.SolidSys(["numspin 1"])
    with pytest.raises(bl.BlochError) as e:
        s.op("Foo")
    assert e.value.status == 1


def test_rotation_matrices_match_reference_formulas():
    a, b, g = 0.3, 1.1, 2.0
    ca, sa, cb, sb, cg, sg = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(g), np.sin(g)
    R3 = np.array([[ca * cb * cg - sa * sg, sa * cb * cg + ca * sg, -sb * cg],
                   [-ca * cb * sg - sa * cg, -sa * cb * sg + ca * cg, sb * sg],
                   [ca * sb, sa * sb, cb]])
    np.testing.assert_allclose(bl.rotationMatrix3D(a, b, g), R3, atol=1e-15)
    R2 = np.array([[np.cos(a), np.sin(a), 0], [-np.cos(b) * np.sin(a), np.cos(a) * np.cos(b), np.sin(b)],
                   [np.sin(a) * np.sin(b), -np.cos(a) * np.sin(b), np.cos(b)]])
    np.testing.assert_allclose(bl.rotationMatrix3D(a, b), R2, atol=1e-15)
    for R in (bl.rotationMatrix3D(a, b, g), bl.rotationMatrix3D(a, b)):
        np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-14)


def test_cpp_host_api_example_builds():
    from blochlib_gb300 import build
    exes = build.build_examples()
    assert exes and all(e.exists() for e in exes)


def _sized(cfg, count=None, **kw):
    s = bl.SolidSys(cfg["lines"])
    phi, theta, gamma, w = (np.asarray(x)[:count] for x in cfg["powder"])
    pw = bl.powder.from_arrays(theta, phi, gamma, w)
    return bl.job_bytes(s, pw, s.op(cfg["rho"]), s.op(cfg["det"]), cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"],
                        **kw)


def test_job_bytes_plans_on_the_host():
    """bl_job_bytes runs without a device: one-warp size <= full size, full size grows by one
    warp's worth per 32 crystallites, the mixed form needs less, bigger systems need more."""
    c1 = W.config(1)
    lo32, hi32 = _sized(c1, 32)
    lo64, hi64 = _sized(c1, 64)
    lo96, hi96 = _sized(c1, 96)
    assert lo32 <= hi32 and lo64 < hi64
    assert hi96 - hi64 == hi64 - hi32 > 0
    assert _sized(c1, 64, precision=1)[1] < hi64
    small, big = _sized(W.config(3, 5), 64), _sized(W.config(3, 0), 64)  # 3 vs 7 protons
    assert big[0] > small[0]


def test_mat5_files_read_back(tmp_path):
    """matstream writes MAT-file level 5 (the reference's Matlab5 format): complex and real
    vectors, matrices, scalars and strings come back exactly through scipy.io.loadmat."""
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(5)
    fid = rng.normal(size=100) + 1j * rng.normal(size=100)
    m = rng.normal(size=(3, 4)) + 1j * rng.normal(size=(3, 4))
    r = rng.normal(size=(2, 5))
    path = tmp_path / "out.mat"
    with bl.matstream(path) as ms:
        ms.put("vdat", fid)
        ms.put("sw1", 123456.5)
        ms.put("mx", m)
        ms.put("rx", r)
        ms.put("note", "powder FID, 3722 crystallites")
    d = sio.loadmat(str(path))
    np.testing.assert_array_equal(d["vdat"], fid.reshape(-1, 1))
    assert d["sw1"].shape == (1, 1) and d["sw1"][0, 0] == 123456.5
    np.testing.assert_array_equal(d["mx"], m)
    np.testing.assert_array_equal(d["rx"], r)
    assert str(d["note"][0]) == "powder FID, 3722 crystallites"
