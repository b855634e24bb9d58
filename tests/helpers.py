"""Test helpers: the CPU oracle (test infrastructure) and job-text plumbing."""
import ctypes
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
_ORACLE = None


def oracle():
    global _ORACLE
    if _ORACLE is None:
        lib = ctypes.CDLL(str(ROOT / "oracle" / "_build" / "liboracle.so"))
        lib.oracle_powder_fid.restype = ctypes.c_int
        lib.oracle_powder_fid.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p]
        _ORACLE = lib
    return _ORACLE


def parse_job(text):
    """job text -> (spin lines, dict of scalar keys)"""
    lines, kv = [], {}
    for raw in str(text).splitlines():
        l = raw.strip()
        if not l or l.startswith("#") or ":" not in l:
            continue
        k, v = l.split(":", 1)
        k, v = k.strip(), v.strip()
        if k == "spin":
            lines.append(v)
        else:
            kv[k] = v
    return lines, kv


def oracle_fid(job_text, rows):
    """rows: C x 4 (phi, theta, gamma, weight).  Returns (fid, sw)."""
    _, kv = parse_job(job_text)
    npts = int(kv["npts"])
    rows = np.ascontiguousarray(np.asarray(rows, dtype=np.float64))
    out = np.zeros(2 * npts)
    sw = np.zeros(1)
    st = oracle().oracle_powder_fid(str(job_text).encode(), rows.ctypes.data, len(rows), out.ctypes.data,
                                    sw.ctypes.data)
    assert st == 0
    return out.view(np.complex128), float(sw[0])


def gpu_fid(job_text, rows, ctx=None, return_sw=False, step_method=None, fave_method=None, precision=0):
    """The CUDA path through the C ABI (oneFID.FID)."""
    import blochlib_gb300 as bl
    lines, kv = parse_job(job_text)
    sys_ = bl.SolidSys(lines)
    if "bfield" in kv:
        sys_.setBfield(float(kv["bfield"]))
    for line in str(job_text).splitlines():  # continuous rf fields, in order
        if line.startswith("rf:"):
            t = line[3:].split()
            sys_.addRf(t[0], float(t[1]), float(t[2]) if len(t) > 2 else 0.0, float(t[3]) if len(t) > 3 else 0.0)
    rows = np.asarray(rows, dtype=np.float64)
    pw = bl.powder.from_arrays(theta=rows[:, 1], phi=rows[:, 0], gamma=rows[:, 2], weight=rows[:, 3])
    drv = bl.oneFID(sys_, int(kv["npts"]), float(kv["sw"]), float(kv["wr"]), float(kv["rotb"]),
                    float(kv.get("start", 0.0)), precision=precision, ctx=ctx, step_method=step_method,
                    fave_method=fave_method)
    if "p2p" in kv:  # point-to-point FID (bl_p2p_fid), with its rf schedule if any
        base, factor = (int(x) for x in kv["p2p"].split())
        sched = []
        for line in str(job_text).splitlines():
            if line.startswith("rfc:"):
                t = line[4:].split()
                sched.append((int(t[0]), t[1], float(t[2]), float(t[3]) if len(t) > 3 else 0.0,
                              float(t[4]) if len(t) > 4 else 0.0))
        fid = drv.p2pFID(pw, sys_.op(kv["rho"]), sys_.op(kv["det"]), base, factor, float(kv.get("maxtstep", 0.0)),
                         rf_chunks=sched)
    else:
        fid = drv.FID(pw, sys_.op(kv["rho"]), sys_.op(kv["det"]))
    return (fid, drv.sw) if return_sw else fid


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if p.stem not in ("zcw_builtin", "hamgen", "plotter_ref"))


def load_golden(name):
    d = np.load(GOLDEN / f"{name}.npz")
    return str(d["job"]), d["powder"], d["fid64"], d["fid32"], float(d["sw"])
