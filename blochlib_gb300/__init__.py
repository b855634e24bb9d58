"""blochlib_gb300: GB300-native powder-averaged MAS spin propagation (gamma-COMPUTE).

Python mirror of BlochLib's host API for the spinning powder-FID path, over the C ABI in
include/blochlib_gb300.h (libblochlib_gb300.so, built in-tree by blochlib_gb300/build.py):

    SolidSys(lines)                    src/QMspins/sys.cc:40-42, read 120-204
    SolidSys.Fx()/Fp()/Ix(k)/...       src/QMspins/spinsys.h:143-162
    powder(powder.zcw, t, p[, g])      src/QMspins/driver/powder.cc:94-113, 248-280
    powder.read(path)                  src/QMspins/driver/powder.cc:333-389
    oneFID(sys, npts, sw, wr, rotb)    src/QMspins/driver/oneFID.h:103-108
    oneFID.FID(powder, ro, det)        src/QMspins/driver/oneFID.h:200-208, 339-431
    plotterFID(fid, file, dt)          src/utils/plotter.cc:49-135

All compute runs in the CUDA library; there is no CPU fallback.  Loading fails loudly
when the library is missing or cannot initialise a GPU.
"""
import ctypes
import math
import os
from pathlib import Path

import numpy as np

__all__ = ["SolidSys", "powder", "oneFID", "PropReduce", "HamiltonianGen", "plotterFID", "Context", "Job", "BlochError", "library_path", "load"]

_HERE = Path(__file__).resolve().parent
_LIB = None


def library_path():
    return _HERE / "libblochlib_gb300.so"


class BlochError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"bl_status {status}: {msg}")
        self.status = status


_SIGS = {
    "bl_last_error": (ctypes.c_char_p, []),
    "bl_last_error_statement": (ctypes.c_double, []),
    "bl_version": (ctypes.c_char_p, []),
    "bl_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_ctx_destroy": (None, [ctypes.c_void_p]),
    "bl_ctx_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "bl_system_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_system_destroy": (None, [ctypes.c_void_p]),
    "bl_system_dim": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_system_spins": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_system_operator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]),
    "bl_system_blocks": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "bl_powder_zcw": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_powder_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_powder_from_arrays": (ctypes.c_int, [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_powder_size": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_powder_get": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "bl_powder_destroy": (None, [ctypes.c_void_p]),
    "bl_powder_fid": (ctypes.c_int, [ctypes.c_void_p] * 8),
    "bl_job_create": (ctypes.c_int, [ctypes.c_void_p] * 6 + [ctypes.POINTER(ctypes.c_void_p)]),
    "bl_p2p_fid": (ctypes.c_int, [ctypes.c_void_p] * 8),
    "bl_server_submit_p2p": (ctypes.c_int, [ctypes.c_void_p] * 6 + [ctypes.POINTER(ctypes.c_longlong)]),
    "bl_hamgen": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "bl_p2p_job_create": (ctypes.c_int, [ctypes.c_void_p] * 6 + [ctypes.POINTER(ctypes.c_void_p)]),
    "bl_job_run": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_job_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "bl_job_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_job_launches": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_job_flops": (ctypes.c_double, [ctypes.c_void_p]),
    "bl_job_tensor_flops": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]),
    "bl_job_sw": (ctypes.c_double, [ctypes.c_void_p]),
    "bl_job_describe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "bl_job_destroy": (None, [ctypes.c_void_p]),
    "bl_plotter_fid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_double]),
    "bl_system_set_bfield": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "bl_system_add_rf": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double]),
    "bl_mat5_open": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_mat5_put": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int]),
    "bl_mat5_put_string": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]),
    "bl_mat5_close": (None, [ctypes.c_void_p]),
    "bl_stage_name": (ctypes.c_char_p, [ctypes.c_int]),
    "bl_job_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "bl_job_stage_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bl_job_stage_flops": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "bl_job_reset_stage_times": (ctypes.c_int, [ctypes.c_void_p]),
    "bl_job_run_timed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "bl_job_io_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
    "bl_probe_fp64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "bl_probe_fp32": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "bl_powder_fid_noalloc": (ctypes.c_int, [ctypes.c_void_p] * 8),
    "bl_rotation3": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "bl_rotation2": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "bl_job_bytes": (ctypes.c_int, [ctypes.c_int] + [ctypes.c_void_p] * 5 + [ctypes.POINTER(ctypes.c_size_t)] * 2),
    "bl_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "bl_server_destroy": (None, [ctypes.c_void_p]),
    "bl_server_submit": (ctypes.c_int, [ctypes.c_void_p] * 6 + [ctypes.POINTER(ctypes.c_longlong)]),
    "bl_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.POINTER(ctypes.c_int),
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bl_server_cancel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong]),
    "bl_server_stats": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_longlong)] * 3 +
                        [ctypes.POINTER(ctypes.c_double)]),
}

STAGES = 8


STEP_EIGH, STEP_TAYLOR = 0, 1


def _step_method(m):
    """Step exponential: 'eigh' (0, Jacobi eigen-decomposition) or 'taylor' (1, faster);
    default from BL_STEP_METHOD, else taylor."""
    if m is None:
        m = os.environ.get("BL_STEP_METHOD", "taylor")
    if isinstance(m, str):
        m = {"eigh": STEP_EIGH, "taylor": STEP_TAYLOR}[m]
    return int(m)


FAVE_AUTO, FAVE_DIRECT, FAVE_FFT = 0, 1, 2


def _fave_method(m):
    """Fave correlation: 'auto' (0), 'direct' (1) or 'fft' (2); default BL_FAVE_METHOD or auto."""
    if m is None:
        m = os.environ.get("BL_FAVE_METHOD", "auto")
    if isinstance(m, str):
        m = {"auto": FAVE_AUTO, "direct": FAVE_DIRECT, "fft": FAVE_FFT}[m]
    return int(m)


class FidParams(ctypes.Structure):
    _fields_ = [("npts", ctypes.c_int), ("sw", ctypes.c_double), ("wr", ctypes.c_double),
                ("rotb_deg", ctypes.c_double), ("start_t", ctypes.c_double), ("precision", ctypes.c_int),
                ("step_method", ctypes.c_int), ("fave_method", ctypes.c_int), ("error_sample", ctypes.c_int)]


class RfChunk(ctypes.Structure):
    _fields_ = [("chunk", ctypes.c_int), ("iso", ctypes.c_char_p), ("amp_hz", ctypes.c_double),
                ("phase_deg", ctypes.c_double), ("offset_hz", ctypes.c_double)]


class P2PParams(ctypes.Structure):
    _fields_ = [("npts", ctypes.c_int), ("sw", ctypes.c_double), ("wr", ctypes.c_double),
                ("rotb_deg", ctypes.c_double), ("start_t", ctypes.c_double), ("precision", ctypes.c_int),
                ("step_method", ctypes.c_int), ("base", ctypes.c_int), ("factor", ctypes.c_int),
                ("maxtstep", ctypes.c_double), ("rf", ctypes.c_void_p), ("nrf", ctypes.c_int)]


def _rf_schedule(rf_chunks):
    """(chunk, iso, amp Hz[, phase deg[, offset Hz]]) tuples -> a ctypes array (kept by the caller)."""
    rows = [tuple(r) + (0.0,) * (5 - len(r)) for r in (rf_chunks or [])]
    arr = (RfChunk * max(1, len(rows)))(*[RfChunk(int(a), str(b).encode(), float(c), float(d), float(e))
                                          for a, b, c, d, e in rows])
    return arr, len(rows)


class HamiltonianGen:
    """HamiltonianGen (src/QMspins/driver/ham_gen.h): operator expressions such as
    "Ix_0 + complexi*Iy_1" or "T2m1_0,1*A21" evaluated to N x N matrices (host side, no GPU)."""

    def __init__(self):
        self.vars = {}

    def addVar(self, name, value):
        self.vars[str(name)] = complex(value)

    def Hamiltonian(self, sys, expr, theta=0.0, phi=0.0, gamma=0.0):
        n = sys.dim()
        out = np.zeros((n, n), dtype=np.complex128)
        names = (ctypes.c_char_p * max(1, len(self.vars)))(*[k.encode() for k in self.vars])
        vals = np.array([[v.real, v.imag] for v in self.vars.values()], dtype=np.float64).reshape(-1)
        _check(load().bl_hamgen(sys._h, str(expr).encode(), float(theta), float(phi), float(gamma),
                                ctypes.cast(names, ctypes.c_void_p), _ptr(vals) if len(vals) else None,
                                len(self.vars), _ptr(out)))
        return out


class PropReduce:
    """PropReduce(base, factor) (examples/qmsims/MMMQMAS/propreduce.cc:16-60): a rotor period
    cut into `base` chunks, one dwell spanning `factor` of them, both divided by their gcd.
    sequences()[k] lists the chunks (in time order) that dwell k mod base covers."""

    def __init__(self, base, factor):
        if int(base) <= 0 or int(factor) <= 0:
            raise ValueError("base and factor must be positive")
        g = math.gcd(int(base), int(factor))
        self.base, self.factor = int(base) // g, int(factor) // g

    def sequences(self):
        b, f = self.base, self.factor
        return [[(k * f + m) % b for m in range(f)] for k in range(b)]


def load():
    """Load the CUDA library (no fallback: raises if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = library_path()
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def _check(st):
    if st != 0:
        raise BlochError(st, load().bl_last_error().decode())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _cmat(m, n):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    if m.shape != (n, n):
        raise ValueError(f"operator must be {n}x{n}, got {m.shape}")
    return m


class Context:
    """One CUDA device + stream (bl_ctx)."""

    def __init__(self, device=0, hbm_budget=0):
        lib = load()
        h = ctypes.c_void_p()
        _check(lib.bl_ctx_create(int(device), int(hbm_budget), ctypes.byref(h)))
        self._h = h

    @property
    def stream(self):
        return load().bl_ctx_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            load().bl_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("BL_DEVICE", "0")))
    return _default_ctx


def probe_fp64_tflops(ctx=None):
    """Measured DFMA throughput of the device (TFLOP/s)."""
    t = ctypes.c_double()
    _check(load().bl_probe_fp64((ctx or default_context())._h, ctypes.byref(t)))
    return t.value


def probe_fp32_tflops(ctx=None):
    """Measured FFMA throughput of the device (TFLOP/s): the FP32 pipe of the mixed form's
    double-float stages."""
    t = ctypes.c_double()
    _check(load().bl_probe_fp32((ctx or default_context())._h, ctypes.byref(t)))
    return t.value


class SolidSys:
    """Spin system from the reference's text format (list of lines or one string)."""

    def __init__(self, lines):
        text = lines if isinstance(lines, str) else "\n".join(lines)
        self.text = text
        lib = load()
        h = ctypes.c_void_p()
        _check(lib.bl_system_create(text.encode(), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                load().bl_system_destroy(self._h)
        except Exception:
            pass

    def setBfield(self, bfield):
        """SolidSys::setBfield: with |B| > 1e-12 quadrupoles add their second-order term
        (or use it alone when their Q line's order column is 2)."""
        _check(load().bl_system_set_bfield(self._h, float(bfield)))

    def addRf(self, iso, amp, phase=0.0, offset=0.0):
        """Continuous rf on every `iso` spin during the FID (solid-2.0 PulseData::Pulse):
        amp (Ix cos phase + Iy sin phase) + offset Iz, Hz and degrees."""
        _check(load().bl_system_add_rf(self._h, str(iso).encode(), float(amp), float(phase), float(offset)))

    def dim(self):
        return load().bl_system_dim(self._h)

    def spins(self):
        return load().bl_system_spins(self._h)

    def blocks(self):
        lib = load()
        n = ctypes.c_int()
        _check(lib.bl_system_blocks(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        _check(lib.bl_system_blocks(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out.tolist()

    def op(self, expr):
        n = self.dim()
        out = np.zeros((n, n), dtype=np.complex128)
        _check(load().bl_system_operator(self._h, expr.encode(), _ptr(out)))
        return out

    # reference accessor names (spinsys.h:143-162)
    def Fx(self): return self.op("Fx")
    def Fy(self): return self.op("Fy")
    def Fz(self): return self.op("Fz")
    def Fp(self): return self.op("Fp")
    def Fmi(self): return self.op("Fm")
    def Fe(self): return self.op("Fe")
    def Ix(self, k): return self.op(f"Ix {k}")
    def Iy(self, k): return self.op(f"Iy {k}")
    def Iz(self, k): return self.op(f"Iz {k}")
    def Ip(self, k): return self.op(f"Ip {k}")
    def Imi(self, k): return self.op(f"Im {k}")


class powder:
    """Powder angle set (theta, phi, gamma, weight), radians."""
    zcw = "zcw"

    def __init__(self, method=None, tstep=0, pstep=0, gstep=0, _handle=None):
        lib = load()
        if _handle is not None:
            self._h = _handle
        elif method == powder.zcw:
            h = ctypes.c_void_p()
            _check(lib.bl_powder_zcw(int(tstep), int(pstep), int(gstep), ctypes.byref(h)))
            self._h = h
        elif isinstance(method, (str, os.PathLike)):
            h = ctypes.c_void_p()
            _check(lib.bl_powder_read(str(method).encode(), ctypes.byref(h)))
            self._h = h
        else:
            raise ValueError("powder(method): use powder.zcw or a powder file path")

    @classmethod
    def read(cls, path):
        return cls(str(path))

    @classmethod
    def from_arrays(cls, theta, phi, gamma, weight):
        th, ph, ga, w = (np.ascontiguousarray(np.asarray(x, dtype=np.float64)) for x in (theta, phi, gamma, weight))
        if not (len(th) == len(ph) == len(ga) == len(w)):
            raise ValueError("powder arrays differ in length")
        h = ctypes.c_void_p()
        _check(load().bl_powder_from_arrays(_ptr(th), _ptr(ph), _ptr(ga), _ptr(w), len(th), ctypes.byref(h)))
        return cls(_handle=h)

    def size(self):
        return load().bl_powder_size(self._h)

    def arrays(self):
        n = self.size()
        out = [np.zeros(n) for _ in range(4)]
        _check(load().bl_powder_get(self._h, *(_ptr(a) for a in out)))
        return tuple(out)  # theta, phi, gamma, weight

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                load().bl_powder_destroy(self._h)
        except Exception:
            pass


class Job:
    """Resident job (bl_job): inputs on the device; run() recomputes the powder FID."""

    def __init__(self, sys, pw, ro, det, npts, sw, wr, rotb, start_t=0.0, precision=0, ctx=None, step_method=None,
                 fave_method=None):
        self.ctx = ctx or default_context()
        n = sys.dim()
        self._ro, self._det = _cmat(ro, n), _cmat(det, n)
        self.params = FidParams(int(npts), float(sw), float(wr), float(rotb), float(start_t), int(precision),
                                _step_method(step_method), _fave_method(fave_method))
        h = ctypes.c_void_p()
        _check(load().bl_job_create(self.ctx._h, sys._h, pw._h, _ptr(self._ro), _ptr(self._det),
                                    ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        self.npts = int(npts)

    @classmethod
    def p2p(cls, sys, pw, ro, det, npts, wr, rotb, base, factor, maxtstep=0.0, sw=0.0, start_t=0.0, precision=0,
            ctx=None, step_method=None, rf_chunks=None):
        """Resident point-to-point job (bl_p2p_job_create); see oneFID.p2pFID."""
        self = cls.__new__(cls)
        self.ctx = ctx or default_context()
        n = sys.dim()
        self._ro, self._det = _cmat(ro, n), _cmat(det, n)
        self._rf, nrf = _rf_schedule(rf_chunks)
        self.params = P2PParams(int(npts), float(sw), float(wr), float(rotb), float(start_t), int(precision),
                                _step_method(step_method), int(base), int(factor), float(maxtstep),
                                ctypes.cast(self._rf, ctypes.c_void_p), nrf)
        h = ctypes.c_void_p()
        _check(load().bl_p2p_job_create(self.ctx._h, sys._h, pw._h, _ptr(self._ro), _ptr(self._det),
                                        ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        self.npts = int(npts)
        return self

    def run(self):
        _check(load().bl_job_run(self._h))

    def read(self):
        out = np.zeros(self.npts, dtype=np.complex128)
        _check(load().bl_job_read(self._h, _ptr(out)))
        return out

    def sync(self):
        _check(load().bl_job_sync(self._h))

    @property
    def launches(self):
        return load().bl_job_launches(self._h)

    @property
    def flops(self):
        return load().bl_job_flops(self._h)

    def tensor_flops(self):
        """(step, Dyson): BF16 tensor-core flops of the last run's exact-slice products."""
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(load().bl_job_tensor_flops(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    @property
    def sw(self):
        return load().bl_job_sw(self._h)

    def set_profiling(self, on=True):
        _check(load().bl_job_set_profiling(self._h, int(bool(on))))

    def stage_times(self):
        """{stage name: (ms accumulated, launches)}"""
        ms = np.zeros(STAGES)
        nl = np.zeros(STAGES, dtype=np.int32)
        _check(load().bl_job_stage_times(self._h, _ptr(ms), _ptr(nl)))
        lib = load()
        return {lib.bl_stage_name(i).decode(): (float(ms[i]), int(nl[i])) for i in range(STAGES)}

    def stage_flops(self):
        f = np.zeros(STAGES)
        _check(load().bl_job_stage_flops(self._h, _ptr(f)))
        lib = load()
        return {lib.bl_stage_name(i).decode(): float(f[i]) for i in range(STAGES)}

    def reset_stage_times(self):
        _check(load().bl_job_reset_stage_times(self._h))

    def run_timed(self, iters):
        ms = ctypes.c_double()
        _check(load().bl_job_run_timed(self._h, int(iters), ctypes.byref(ms)))
        return ms.value

    def io_bytes(self):
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        _check(load().bl_job_io_bytes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def describe(self):
        import json
        buf = ctypes.create_string_buffer(4096)
        load().bl_job_describe(self._h, buf, 4096)
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None):
            load().bl_job_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class oneFID:
    """oneFID<SolidSys>(sys, npts, sw, wr, rotb_deg, startT)  (oneFID.h:103-108)."""

    def __init__(self, sys, npts, sw=20000.0, wr=0.0, rotb=0.0, startT=0.0, precision=0, ctx=None, step_method=None,
                 fave_method=None, error_sample=0):
        self.sys, self.npts, self.sw, self.wr, self.rotb, self.startT = sys, int(npts), float(sw), float(wr), float(rotb), float(startT)
        self.precision = precision
        # mixed form: crystallites on which FID() restates the result against FP64 (error_statement)
        self.error_sample = int(error_sample)
        self.error_statement = None
        self.step_method = step_method
        self.fave_method = fave_method
        self.ctx = ctx
        self.fid_ = np.zeros(self.npts, dtype=np.complex128)

    def FID(self, pw, ro, det):
        """Powder-summed FID, sum_c w_c FID_c (oneFID.h:200-208); updates self.sw to n*wr."""
        ctx = self.ctx or default_context()
        n = self.sys.dim()
        ro, det = _cmat(ro, n), _cmat(det, n)
        out = np.zeros(self.npts, dtype=np.complex128)
        sw_out = np.zeros(1)
        params = FidParams(self.npts, self.sw, self.wr, self.rotb, self.startT, int(self.precision),
                           _step_method(self.step_method), _fave_method(self.fave_method), self.error_sample)
        _check(load().bl_powder_fid(ctx._h, self.sys._h, pw._h, _ptr(ro), _ptr(det), ctypes.byref(params),
                                    _ptr(out), _ptr(sw_out)))
        stmt = load().bl_last_error_statement()
        self.error_statement = stmt if stmt >= 0 else None
        self.sw = float(sw_out[0])
        self.fid_ = out
        return out

    def p2pFID(self, pw, ro, det, base=1, factor=1, maxtstep=0.0, rf_chunks=None):
        """Point-to-point powder FID (bl_p2p_fid): points every factor/base rotor periods
        (PropReduce(base, factor)), fid[p] = sum_c w_c Tr(rho_c(t_p) det) / Tr(det det^H);
        steps of at most maxtstep inside each chunk.  Static (wr == 0 or rotor angle 0): one
        step of 1/sw per point.  rf_chunks: (chunk, iso, amp[, phase[, offset]]) fields on
        during one chunk of every rotor period.  Updates self.sw to base*wr/factor."""
        if isinstance(base, PropReduce):
            base, factor = base.base, base.factor
        ctx = self.ctx or default_context()
        n = self.sys.dim()
        ro, det = _cmat(ro, n), _cmat(det, n)
        out = np.zeros(self.npts, dtype=np.complex128)
        sw_out = np.zeros(1)
        rf, nrf = _rf_schedule(rf_chunks)
        params = P2PParams(self.npts, self.sw, self.wr, self.rotb, self.startT, int(self.precision),
                           _step_method(self.step_method), int(base), int(factor), float(maxtstep),
                           ctypes.cast(rf, ctypes.c_void_p), nrf)
        _check(load().bl_p2p_fid(ctx._h, self.sys._h, pw._h, _ptr(ro), _ptr(det), ctypes.byref(params),
                                 _ptr(out), _ptr(sw_out)))
        self.sw = float(sw_out[0])
        self.fid_ = out
        return out


def job_bytes(sys, pw, ro, det, npts, sw, wr, rotb, start_t=0.0, precision=0, step_method=None, fave_method=None,
              device=0):
    """(min_bytes, full_bytes): device memory of the job with 32 crystallites per batch and
    with all crystallites in one batch (bl_job_bytes; host-side planning only)."""
    n = sys.dim()
    ro, det = _cmat(ro, n), _cmat(det, n)
    p = FidParams(int(npts), float(sw), float(wr), float(rotb), float(start_t), int(precision),
                  _step_method(step_method), _fave_method(fave_method))
    lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
    _check(load().bl_job_bytes(int(device), sys._h, pw._h, _ptr(ro), _ptr(det), ctypes.byref(p), ctypes.byref(lo),
                               ctypes.byref(hi)))
    return lo.value, hi.value


class Server:
    """Serving loop with continuous batching (bl_server): `lanes` CUDA streams sharing one
    pool of device memory; requests are sized at submit() and admitted first come first
    served by free memory; poll()/result() collect the FID and latency."""
    QUEUED, RUNNING, DONE, FAILED, CANCELLED = 0, 1, 2, 3, 4

    def __init__(self, device=0, lanes=8, pool_bytes=16 << 30):
        h = ctypes.c_void_p()
        _check(load().bl_server_create(int(device), int(lanes), int(pool_bytes), ctypes.byref(h)))
        self._h = h
        self._npts = {}
        # stated error of the last finished request result() returned (mixed form with
        # error_sample > 0), else None
        self.last_error_statement = None

    def submit(self, sys, pw, ro, det, npts, sw, wr, rotb, start_t=0.0, precision=0, step_method=None,
               fave_method=None, error_sample=0):
        n = sys.dim()
        ro, det = _cmat(ro, n), _cmat(det, n)
        p = FidParams(int(npts), float(sw), float(wr), float(rotb), float(start_t), int(precision),
                      _step_method(step_method), _fave_method(fave_method), int(error_sample))
        t = ctypes.c_longlong()
        _check(load().bl_server_submit(self._h, sys._h, pw._h, _ptr(ro), _ptr(det), ctypes.byref(p), ctypes.byref(t)))
        self._npts[t.value] = int(npts)
        return t.value

    def submit_p2p(self, sys, pw, ro, det, npts, wr, rotb, base, factor, maxtstep=0.0, sw=0.0, start_t=0.0,
                   precision=0, step_method=None, rf_chunks=None):
        """A point-to-point FID request (bl_server_submit_p2p; see oneFID.p2pFID)."""
        n = sys.dim()
        ro, det = _cmat(ro, n), _cmat(det, n)
        rf, nrf = _rf_schedule(rf_chunks)
        p = P2PParams(int(npts), float(sw), float(wr), float(rotb), float(start_t), int(precision),
                      _step_method(step_method), int(base), int(factor), float(maxtstep),
                      ctypes.cast(rf, ctypes.c_void_p), nrf)
        t = ctypes.c_longlong()
        _check(load().bl_server_submit_p2p(self._h, sys._h, pw._h, _ptr(ro), _ptr(det), ctypes.byref(p),
                                           ctypes.byref(t)))
        self._npts[t.value] = int(npts)
        return t.value

    def state(self, ticket):
        st = ctypes.c_int()
        _check(load().bl_server_poll(self._h, int(ticket), ctypes.byref(st), None, None, None))
        return st.value

    def result(self, ticket):
        """(state, fid, sw, latency_ms) once finished (releases the ticket), else (state, None, None, None)."""
        st = ctypes.c_int()
        fid = np.zeros(self._npts[ticket], dtype=np.complex128)
        sw, lat = ctypes.c_double(), ctypes.c_double()
        _check(load().bl_server_poll(self._h, int(ticket), ctypes.byref(st), _ptr(fid), ctypes.byref(sw),
                                     ctypes.byref(lat)))
        if st.value >= self.DONE:
            self._npts.pop(ticket, None)
            if st.value == self.FAILED:
                raise BlochError(5, load().bl_last_error().decode())
            if st.value == self.DONE:
                stmt = load().bl_last_error_statement()
                self.last_error_statement = stmt if stmt >= 0 else None
            return st.value, (fid if st.value == self.DONE else None), sw.value, lat.value
        return st.value, None, None, None

    def cancel(self, ticket):
        _check(load().bl_server_cancel(self._h, int(ticket)))

    def stats(self):
        """(queued, running, finished, algorithmic flop of the completed jobs)."""
        q, r, d, f = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_double()
        _check(load().bl_server_stats(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(d), ctypes.byref(f)))
        return q.value, r.value, d.value, f.value

    def close(self):
        if getattr(self, "_h", None):
            load().bl_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rotationMatrix3D(a, b, g=None):
    """Cartesian rotation of the reference: (alpha, beta, gamma) or the rotor's (phi, theta)."""
    R = np.zeros(9)
    if g is None:
        _check(load().bl_rotation2(float(a), float(b), _ptr(R)))
    else:
        _check(load().bl_rotation3(float(a), float(b), float(g), _ptr(R)))
    return R.reshape(3, 3)


class matstream:
    """MAT-file level 5 output, as the reference's Matlab5 / matstream (bl_mat5_*):
    put(name, value) appends a scalar (1 x 1), a 1-D array (column vector, the reference's
    put(name, Vector)), a 2-D array, real or complex, or a string."""

    def __init__(self, path):
        h = ctypes.c_void_p()
        _check(load().bl_mat5_open(str(path).encode(), ctypes.byref(h)))
        self._h = h

    def put(self, name, value):
        if isinstance(value, str):
            _check(load().bl_mat5_put_string(self._h, name.encode(), value.encode()))
            return
        a = np.asarray(value)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        elif a.ndim == 1:
            a = a.reshape(-1, 1)
        elif a.ndim != 2:
            raise ValueError("matstream.put takes scalars, vectors, matrices or strings")
        cplx = np.iscomplexobj(a)
        d = np.ascontiguousarray(a, dtype=np.complex128 if cplx else np.float64)
        _check(load().bl_mat5_put(self._h, name.encode(), _ptr(d), d.shape[0], d.shape[1], int(cplx)))

    def close(self):
        if getattr(self, "_h", None):
            load().bl_mat5_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plotterFID(fid, datasave="fid", dt=1.0):
    """7-column text file t, f, Re S, Im S, Re fid, Im fid, |S| (plotter.cc:49-135)."""
    f = np.ascontiguousarray(np.asarray(fid, dtype=np.complex128))
    _check(load().bl_plotter_fid(_ptr(f), len(f), str(datasave).encode(), float(dt)))
    return str(datasave)
