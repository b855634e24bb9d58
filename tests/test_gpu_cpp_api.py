"""The C++ host API (include/blochlib_gb300.hpp) end to end: the example program runs a
BlochLib-style powder FID; its plotterFID text matches the Python path to the text's
precision and its MAT-5 output (matstream) bit for bit."""
import subprocess

import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import build

pytestmark = pytest.mark.gpu


def test_cpp_example_matches_python_path(tmp_path):
    exe = [e for e in build.build_examples() if e.name == "mas_powder_fid"][0]
    out = tmp_path / "fid.txt"
    npts, sw, wr, beta, t, p = 256, 40 * 15000.0, 15000.0, 54.7356, 144, 89
    r = subprocess.run([str(exe), str(npts), str(sw), str(wr), str(beta), str(t), str(p), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = np.loadtxt(out)
    spinl = ["numspin 3", "T 1H 0", "T 1H 1", "T 1H 2",
             "C 1243 1548 0.3 0 10 20 30", "C -4561 3215 0.5 1 40 50 60", "C 200 2500 0.1 2 70 80 90",
             "D -12000 0 1 0 30 0", "D -7000 1 2 45 60 0", "D -5000 0 2 90 100 0", "J 120 0 1"]
    s = bl.SolidSys(spinl)
    fid = bl.oneFID(s, npts, sw, wr, beta).FID(bl.powder(bl.powder.zcw, t, p), s.Fx() + s.Fz(), s.Fp())
    np.testing.assert_allclose(d[:npts, 4] + 1j * d[:npts, 5], fid, rtol=2e-5, atol=2e-5 * np.abs(fid).max())
    sio = pytest.importorskip("scipy.io")
    m = sio.loadmat(str(out) + ".mat")
    np.testing.assert_array_equal(m["vdat"][:, 0], fid)
    assert m["sw1"][0, 0] == sw


def test_cpp_decoupled_p2p_example_matches_python_path(tmp_path):
    """HamiltonianGen, addRf, PropReduce and p2pFID of the C++ mirror against the same calls
    through the Python mirror: the same engine, so the FIDs agree bit for bit."""
    exe = [e for e in build.build_examples() if e.name == "decoupled_p2p"][0]
    out = tmp_path / "dec.mat"
    npts, wr, amp, ph, t, p = 128, 12000.0, 70000.0, 30.0, 144, 89
    r = subprocess.run([str(exe), str(npts), str(wr), str(amp), str(ph), str(t), str(p), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    sio = pytest.importorskip("scipy.io")
    m = sio.loadmat(str(out))
    spinl = ["numspin 3", "T 13C 0", "T 1H 1", "T 1H 2", "C 1500 6000 0.5 0 10 70 30", "D 8000 0 1 20 30 40",
             "D 5000 0 2 60 10 0", "D -18000 1 2 70 80 0"]
    s = bl.SolidSys(spinl)
    s.addRf("1H", amp, ph)
    g = bl.HamiltonianGen()
    ro, det = g.Hamiltonian(s, "Ix_0"), g.Hamiltonian(s, "Ip_0")
    np.testing.assert_array_equal(m["ro"], ro)
    pw = bl.powder(bl.powder.zcw, t, p)
    drv = bl.oneFID(s, npts, 40 * wr, wr, 54.7356, step_method="taylor")
    np.testing.assert_array_equal(m["fid"][:, 0], drv.FID(pw, ro, det))
    assert m["sw"][0, 0] == drv.sw
    np.testing.assert_array_equal(m["p2p"][:, 0], drv.p2pFID(pw, ro, det, bl.PropReduce(18, 14), maxtstep=2e-6))
    assert m["sw_p2p"][0, 0] == drv.sw == wr * 9 / 7
