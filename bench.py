#!/usr/bin/env python3
"""Benchmark: powder FIDs/s of the spinning powder-FID path on one GB300.

A step is one powder-averaged FID of the workload (default c1: 4 x 1H, dim 16, 3722 ZCW
crystallites, 128 steps per rotor period, 2048 points; blochlib_gb300/workloads.py).

  value     FIDs/s with every input resident in HBM (bl_job_run), CUDA events on the
            engine's stream around exactly K steps, max over ranks.
  e2e       FIDs/s through the reference-facing call (bl_powder_fid: host buffers in,
            upload, compute, FID read back), wall clock around K calls.
  roofline  the stage with the largest share of the timed region: its algorithmic FP64
            flop per run / its CUDA-event time per run, against the DFMA peak measured
            live by the engine's probe kernel.
  cpu_baseline  the reference's own CPU path (oracle/_ref/ref_fid, as shipped), one
            process per host core over contiguous crystallite ranges, on a bounded sample,
            scaled to FIDs/s; the CPU restatement (oracle) where the reference binary is
            absent.

--impl reference times only that CPU path (rank 0), on the same workload and metric.
Multi-GPU: crystallites are independent, so N ranks run N replicas (weak scaling) with no
data-path collective; torch.distributed (gloo) is used only for the barrier and the max.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "powder FIDs/s & p50/p99 latency, mixed vs FP64 GPU path at ≤1e-6 rel err"
UNIT = "powder FIDs/s"
# the mixed form's arithmetic: step and Dyson in double-float (hi + lo floats) on the FP32 pipe,
# Floquet eigenvalues/vectors and the powder sum in FP64, eigenframe, Q/R, Fave and FID terms in FP32
MIXED_DTYPE = "f64+df32+f32 (double-float: step, Dyson; f64: Floquet, powder sum; f32: eigenframe, Q/R, Fave, FID)"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Dist:
    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())


class Clocks:
    """nvidia-smi sampler (every 200 ms) around the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.proc, self.lines = device, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(args):
    """The single-job workload: c0/c1/c2, or one seeded c3/c4 system (--system), with
    optional overrides of the steps per rotor period (--period-steps)."""
    from blochlib_gb300 import workloads as W
    idx = {"c0": 0, "c1": 1, "c2": 2, "c3": 3, "c4": 4}[args.config]
    cfg = W.config(idx, args.system or 0)
    if args.period_steps:
        cfg = dict(cfg, sw=args.period_steps * cfg["wr"])
    if args.p2p:  # point-to-point FID: a point every factor/base rotor periods
        cfg = dict(cfg, p2p=(args.p2p[0], args.p2p[1], args.maxtstep))
    return cfg


def job_text(cfg):
    """The workload in the reference harness's job format (with its p2p line if any)."""
    from blochlib_gb300 import workloads as W
    t = W.job_text(cfg)
    if "p2p" in cfg:
        b, f, mt = cfg["p2p"]
        t += f"p2p: {b} {f}\nmaxtstep: {mt!r}\n"
    return t


def describe(cfg, dim):
    if "p2p" in cfg:
        b, f, mt = cfg["p2p"]
        return (f"point-to-point every {f}/{b} rotor periods, chunks of ceil(1/(wr*{b})/{mt:g} s) steps"
                if mt > 0 else f"point-to-point every {f}/{b} rotor periods, one step per chunk")
    return f"n={int(round(cfg['sw'] / cfg['wr']))} steps/period"


def drive_fid(bl, cfg, drv, pw, ro, det):
    """The reference-facing call: oneFID::FID, or p2pFID for a point-to-point workload."""
    if "p2p" in cfg:
        b, f, mt = cfg["p2p"]
        return drv.p2pFID(pw, ro, det, b, f, mt)
    return drv.FID(pw, ro, det)


def make_job(bl, cfg, ctx, step_method=None, fave_method=None, precision=0):
    s = bl.SolidSys(cfg["lines"])
    phi, theta, gamma, w = cfg["powder"]
    pw = bl.powder.from_arrays(theta, phi, gamma, w)
    ro, det = s.op(cfg["rho"]), s.op(cfg["det"])
    if "p2p" in cfg:
        b, f, mt = cfg["p2p"]
        job = bl.Job.p2p(s, pw, ro, det, cfg["npts"], cfg["wr"], cfg["rotb"], b, f, maxtstep=mt, sw=cfg["sw"],
                         ctx=ctx, step_method=step_method, precision=precision)
    else:
        job = bl.Job(s, pw, ro, det, cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], ctx=ctx,
                     step_method=step_method, fave_method=fave_method, precision=precision)
    return s, pw, ro, det, job


# ------------------------------------------------------------------ CPU baseline
def _ref_binary():
    ref = ROOT / "oracle" / "_ref" / "ref_fid"
    if ref.exists() and os.access(ref, os.X_OK):
        return ref, "reference"
    port = ROOT / "oracle" / "_build" / "gcompute_ref"
    if not port.exists():
        from blochlib_gb300 import build
        build.build_oracle()
    return port, "port"


def _cpu_run(binary, cfg, ranges, tmp):
    """Runs one process per (start, count) range concurrently; returns wall seconds."""
    from blochlib_gb300 import workloads as W
    phi, theta, gamma, w = cfg["powder"]
    procs = []
    t0 = time.perf_counter()
    for i, (a, k) in enumerate(ranges):
        pf = Path(tmp) / f"pw{i}.txt"
        with open(pf, "w") as f:
            for j in range(a, a + k):
                f.write(f"{phi[j]:.17g} {theta[j]:.17g} {gamma[j]:.17g} {w[j]:.17g}\n")
        jf = Path(tmp) / f"job{i}.txt"
        jf.write_text(job_text(cfg) + f"powder: {pf}\n")
        procs.append(subprocess.Popen([str(binary), str(jf), str(Path(tmp) / f"out{i}.bin")],
                                      stdout=subprocess.DEVNULL, stderr=subprocess.PIPE))
    for p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("CPU baseline process failed: " + err.decode()[-500:])
    return time.perf_counter() - t0


def cpu_baseline(cfg, target_s=15.0, cores=None):
    binary, kind = _ref_binary()
    cores = cores or os.cpu_count() or 1
    C = len(cfg["powder"][0])
    with tempfile.TemporaryDirectory() as tmp:
        t2 = _cpu_run(binary, cfg, [(0, 2)], tmp)
        per = max(t2 / 2, 1e-4)
        k = int(max(1, min(C // cores, round(target_s / per))))
        ranges = [(i * k % max(C - k, 1), k) for i in range(cores)]
        wall = _cpu_run(binary, cfg, ranges, tmp)
    fids = cores * k / C
    return {"value": fids / wall, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{cores} processes x {k} crystallites ({cores * k} of {C}) of the full workload, "
                      f"{wall:.1f} s wall, scaled to powder FIDs/s",
            "binary": str(binary.relative_to(ROOT))}


# ------------------------------------------------------------------ main
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cfg = workload(args)
    binary, kind = _ref_binary()
    vals = []
    # each step is a bounded sample; the whole run stays within about two minutes
    step_s = max(1.0, min(args.cpu_seconds, 120.0 / max(args.steps, 1)))
    for i in range(args.warmup):
        cpu_baseline(cfg, target_s=1.0)
    for i in range(args.steps):
        vals.append(cpu_baseline(cfg, target_s=step_s)["value"])
    v = statistics.median(vals)
    last = cpu_baseline(cfg, target_s=1.0)
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, workloads.py)",
           "config": {"workload": f"{cfg['name']}: {cfg['lines'][0]}, dim {2 ** int(cfg['lines'][0].split()[1])}, "
                                  f"{len(cfg['powder'][0])} crystallites, {describe(cfg, 0)}, "
                                  f"npts={cfg['npts']}"},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": last["cores"], "kind": kind,
                            "sample": f"per step: {last['cores']} processes, contiguous crystallite ranges, "
                                      f"~{args.cpu_seconds:.0f} s of CPU work, scaled to powder FIDs/s"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ------------------------------------------------------------------ batching and serving forms
def _job_inputs(bl, cfg):
    s = bl.SolidSys(cfg["lines"])
    phi, theta, gamma, w = cfg["powder"]
    pw = bl.powder.from_arrays(theta, phi, gamma, w)
    return dict(sys=s, pw=pw, ro=s.op(cfg["rho"]), det=s.op(cfg["det"]), npts=cfg["npts"], sw=cfg["sw"],
                wr=cfg["wr"], rotb=cfg["rotb"])


def _drain(srv, tickets, timeout):
    """Polls until every ticket finished or timeout; returns {ticket: (state, fid, latency)}."""
    out, t0 = {}, time.perf_counter()
    pending = list(tickets)
    while pending and time.perf_counter() - t0 < timeout:
        pending = [t for t in pending if not _collect(srv, t, out)]
        if pending:
            time.sleep(0.001)
    return out, pending


def _collect(srv, t, out):
    """Stores (state, fid, latency_ms) of a finished ticket in out; False while it runs."""
    if srv.state(t) < srv.DONE:
        return False
    import blochlib_gb300 as bl
    try:
        st, fid, _, lat = srv.result(t)
    except bl.BlochError:
        st, fid, lat = srv.FAILED, None, None
    out[t] = (st, fid, lat)
    return True


def run_batch(args):
    """c3: a set of seeded spin systems (2..7 1H, n 64..256, 1024 points, powders of 144..1154)
    submitted at once to the serving loop; FIDs/s of the whole batch, mixed and FP64."""
    import blochlib_gb300 as bl
    from blochlib_gb300 import workloads as W
    rank, world, local = dist_env()
    cfgs = [W.config(3, i) for i in range(args.systems)]
    jobs = [_job_inputs(bl, c) for c in cfgs]
    peak = bl.probe_fp64_tflops(bl.Context(local))
    clocks = Clocks(local)
    clocks.start()
    forms, fids = {}, {}
    for prec in ("mixed", "fp64"):
        srv = bl.Server(local, lanes=args.lanes, pool_bytes=args.pool_gib << 30)
        warm = srv.submit(**jobs[0], precision=1 if prec == "mixed" else 0, step_method="taylor")
        _drain(srv, [warm], 300)
        flops0 = srv.stats()[3]
        t0 = time.perf_counter()
        tickets = [srv.submit(**j, precision=1 if prec == "mixed" else 0, step_method="taylor") for j in jobs]
        res, pending = _drain(srv, tickets, 3600)
        dt = time.perf_counter() - t0
        flops = srv.stats()[3] - flops0
        ok = [t for t in tickets if t in res and res[t][0] == srv.DONE]
        lat = [res[t][2] for t in ok]
        forms[prec] = {"fids_per_s": len(ok) / dt, "seconds": dt, "completed": len(ok), "failed": len(tickets) - len(ok),
                       "tflops_algorithmic": flops / dt / 1e12,
                       "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}}
        fids[prec] = [res[t][1] for t in tickets]
        srv.close()
    clk = clocks.stop()
    errs = [_rel(a, b) for a, b in zip(fids["mixed"], fids["fp64"]) if a is not None and b is not None]
    forms["mixed"]["rel_err_vs_fp64_max"] = max(errs) if errs else None
    forms["mixed_speedup_vs_fp64"] = forms["mixed"]["fids_per_s"] / forms["fp64"]["fids_per_s"]
    if rank != 0:
        return 0
    dims = sorted({2 ** int(c["lines"][0].split()[1]) for c in cfgs})
    print(json.dumps({
        "metric": METRIC, "value": forms["mixed"]["fids_per_s"], "unit": UNIT, "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": 1e3 * forms["mixed"]["seconds"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": MIXED_DTYPE, "data": "synthetic (seeded, workloads.py config 3)",
        "config": {"workload": f"c3 batching form: {len(cfgs)} seeded systems, dims {dims}, n 64-256, 1024 points, "
                               "powders 144/320/678/1154, all submitted at once", "lanes": args.lanes,
                   "pool_gib": args.pool_gib, "precision": "mixed (FP64 row for comparison)"},
        "latency_ms": forms["mixed"]["latency_ms"], "precision_forms": forms,
        "roofline": {"bound": "fp64", "kernel": "whole batch (all stages)", "form": "fp64",
                     "achieved": forms["fp64"]["tflops_algorithmic"], "peak": peak, "unit": "TFLOP/s",
                     "frac": forms["fp64"]["tflops_algorithmic"] / peak if peak else None, "traffic": None,
                     "peak_source": "measured live: DFMA probe kernel"},
        "clocks": clk}))
    return 0


def run_serving(args):
    """c4: Poisson request stream (seeded) of c3-like jobs plus 10% large jobs (9-10 x 1H,
    dims 512-1024, on the 100-point repulsion set), for a fixed window; the backlog left at
    the end is cancelled and reported.  Mixed and FP64 on the same stream."""
    import blochlib_gb300 as bl
    from blochlib_gb300 import workloads as W
    rank, world, local = dist_env()
    rng = np.random.default_rng(W.SEED0 + 4)
    small = [_job_inputs(bl, W.config(3, 1000 + i)) for i in range(48)]
    large = [_job_inputs(bl, W.config(4, i)) for i in range(4)]
    n_req = int(args.rate * args.duration)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n_req))
    picks = [(large[rng.integers(len(large))] if rng.uniform() < 0.1 else small[rng.integers(len(small))])
             for _ in range(n_req)]
    forms = {}
    for prec in ("mixed", "fp64"):
        srv = bl.Server(local, lanes=args.lanes, pool_bytes=args.pool_gib << 30)
        warm = srv.submit(**small[0], precision=1 if prec == "mixed" else 0, step_method="taylor")
        _drain(srv, [warm], 300)
        t0 = time.perf_counter()
        done, open_ = {}, []
        i = 0
        while i < n_req:
            now = time.perf_counter() - t0
            while i < n_req and arrivals[i] <= now:
                open_.append(srv.submit(**picks[i], precision=1 if prec == "mixed" else 0, step_method="taylor"))
                i += 1
            open_ = [t for t in open_ if not _collect(srv, t, done)]
            time.sleep(0.0005)
        window = time.perf_counter() - t0
        drained, pending = _drain(srv, open_, args.drain)
        done.update(drained)
        cancelled = 0
        for t in pending:
            try:
                srv.cancel(t)
                cancelled += 1
            except bl.BlochError:
                pass  # already running: it finishes below
        late, _ = _drain(srv, pending, 600)
        total = time.perf_counter() - t0
        ok = [v[2] for v in done.values() if v[0] == srv.DONE]
        forms[prec] = {"offered_per_s": args.rate, "submitted": n_req, "completed": len(ok),
                       "cancelled_backlog": cancelled,
                       "finished_after_drain": sum(v[0] == srv.DONE for v in late.values()), "achieved_fids_per_s": len(ok) / total,
                       "window_s": window, "total_s": total,
                       "latency_ms": {"p50": float(np.percentile(ok, 50)) if ok else None,
                                      "p99": float(np.percentile(ok, 99)) if ok else None}}
        srv.close()
    forms["mixed_speedup_vs_fp64"] = forms["mixed"]["achieved_fids_per_s"] / forms["fp64"]["achieved_fids_per_s"]
    if rank != 0:
        return 0
    print(json.dumps({
        "metric": METRIC, "value": forms["mixed"]["achieved_fids_per_s"], "unit": UNIT, "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": 1e3 * forms["mixed"]["total_s"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": MIXED_DTYPE, "data": "synthetic seeded Poisson stream (workloads.py)",
        "config": {"workload": f"c4 serving form: Poisson {args.rate}/s for {args.duration} s, 90% c3-like, 10% "
                               "9-10 x 1H (dims 512-1024) on rep100", "lanes": args.lanes, "pool_gib": args.pool_gib,
                   "drain_s": args.drain},
        "latency_ms": forms["mixed"]["latency_ms"], "precision_forms": forms}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2", "c3", "c4"])
    ap.add_argument("--systems", type=int, default=128, help="c3: number of seeded systems in the batch")
    ap.add_argument("--system", type=int, default=None,
                    help="c3/c4: time this one seeded system as a single job instead of the batching/serving form")
    ap.add_argument("--period-steps", type=int, default=0, help="override the steps per rotor period (sw = n wr)")
    ap.add_argument("--lanes", type=int, default=16, help="c3/c4: serving lanes (CUDA streams)")
    ap.add_argument("--pool-gib", type=int, default=128, help="c3/c4: serving memory pool (GiB)")
    ap.add_argument("--rate", type=float, default=200.0, help="c4: offered requests per second")
    ap.add_argument("--duration", type=float, default=10.0, help="c4: arrival window (s)")
    ap.add_argument("--drain", type=float, default=20.0, help="c4: wait after the window (s)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--p2p", type=int, nargs=2, default=None, metavar=("BASE", "FACTOR"),
                    help="point-to-point FID every FACTOR/BASE rotor periods instead of gamma-COMPUTE")
    ap.add_argument("--maxtstep", type=float, default=0.0, help="--p2p: longest step inside a chunk (s)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--crystallites", type=int, default=0,
                    help="use only the first N crystallites (smaller case for profiler captures)")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"],
                    help="path timed for 'value' (default: fp64 for c0/c1, mixed for c2)")
    ap.add_argument("--no-compare", action="store_true", help="skip the other precision form")
    ap.add_argument("--fave-method", default=None, choices=["auto", "direct", "fft"])
    ap.add_argument("--step-method", default="taylor", choices=["eigh", "taylor"],
                    help="FP64 step exponential (default taylor: the faster exact form)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c3" and args.system is None:
        return run_batch(args)
    if args.config == "c4" and args.system is None:
        return run_serving(args)
    args.warmup = max(args.warmup, 3)
    prec = args.precision or ("mixed" if args.config == "c2" else "fp64")
    import blochlib_gb300 as bl
    d = Dist()
    ctx = bl.Context(d.local)
    cfg = workload(args)
    if args.crystallites:
        cfg = dict(cfg, powder=tuple(np.asarray(x)[:args.crystallites] for x in cfg["powder"]))
    s, pw, ro, det, job = make_job(bl, cfg, ctx, args.step_method, args.fave_method, 1 if prec == "mixed" else 0)
    for _ in range(args.warmup):
        job.run()
    job.sync()
    peak = bl.probe_fp64_tflops(ctx)
    clocks = Clocks(d.local)
    clocks.start()
    time.sleep(0.5)
    job.set_profiling(True)
    job.reset_stage_times()
    d.barrier()
    job.sync()
    per_step = [job.run_timed(1) for _ in range(args.steps)]
    job.sync()
    d.barrier()
    ms_total = sum(per_step)
    clk = clocks.stop()
    ms_max = d.max(ms_total)
    value = d.world * args.steps / (ms_max / 1e3)
    fid_main = job.read()
    stages = job.stage_times()
    sflops = job.stage_flops()
    if "p2p" in cfg:  # stage 5 runs the point-to-point terms instead of the Fave correlation
        stages = {("k_p2p_elems" if k == "k_fave" else k): v for k, v in stages.items()}
        sflops = {("k_p2p_elems" if k == "k_fave" else k): v for k, v in sflops.items()}
    dom = max(stages, key=lambda k: stages[k][0])
    dom_ms_per_run = stages[dom][0] / args.steps
    achieved = sflops[dom] / (dom_ms_per_run / 1e3) / 1e12
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(args.config, {}).get(dom)
        except (ValueError, AttributeError):
            traffic = None
    launches_per_run = job.launches
    job.set_profiling(False)
    forms = {prec: {"fids_per_s": value, "ms_per_fid": ms_max / args.steps}}
    if not args.no_compare:
        other = "fp64" if prec == "mixed" else "mixed"
        _, _, _, _, job2 = make_job(bl, cfg, ctx, args.step_method, args.fave_method, 1 if other == "mixed" else 0)
        job2.run()
        job2.sync()
        k2 = max(1, min(args.steps, 10))
        ms2 = job2.run_timed(k2) / k2
        fid_other = job2.read()
        forms[other] = {"fids_per_s": 1e3 / ms2, "ms_per_fid": ms2}
        f64, fmx = (fid_main, fid_other) if prec == "fp64" else (fid_other, fid_main)
        forms["mixed"]["rel_err_vs_fp64"] = _rel(fmx, f64)
        forms["mixed_speedup_vs_fp64"] = forms["mixed"]["fids_per_s"] / forms["fp64"]["fids_per_s"]
        job2.close()
    # e2e through the reference-facing call with host buffers
    drv = bl.oneFID(s, cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], ctx=ctx, step_method=args.step_method,
                    fave_method=args.fave_method, precision=1 if prec == "mixed" else 0)
    drive_fid(bl, cfg, drv, pw, ro, det)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        drive_fid(bl, cfg, drv, pw, ro, det)
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    h2d, d2h = job.io_bytes()
    h2d += 8 * 4 * len(cfg["powder"][0]) + 2 * ro.nbytes  # the caller's powder arrays and rho/det
    if d.rank != 0:
        return 0
    dtype = "f64" if prec == "fp64" else MIXED_DTYPE
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": d.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded spin systems and ZCW powder, workloads.py)",
        "config": {"workload": f"{cfg['name']}: {cfg['lines'][0]} ({' '.join(cfg['lines'][1:2])}...), "
                               f"dim {s.dim()}, {len(cfg['powder'][0])} crystallites, "
                               f"{describe(cfg, s.dim())}, npts={cfg['npts']}, "
                               f"{'plain FP64' if prec == 'fp64' else 'mixed precision'}",
                   "precision": prec, "step_method": args.step_method,
                   "parallelism": f"replicas x{d.world}",
                   "l2": "inputs larger than L2: each step streams the per-crystallite work buffers (GBs)",
                   "layout": job.describe()},
        "latency_ms": {"p50": float(np.percentile(per_step, 50)), "p99": float(np.percentile(per_step, 99))},
        "precision_forms": forms,
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "peak_source": "measured live: DFMA probe kernel (MEASURED_PEAKS.json has no FP64 figure)",
                     "stage_share": {k: v[0] / ms_total for k, v in stages.items()}},
        "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches_per_run * args.steps,
        "clocks": clk,
    }
    if prec == "mixed":  # the step and Dyson run double-float on the FP32 pipe, Floquet on the FP64 pipe
        out["roofline"]["form"] = "mixed"
        out["roofline"]["note"] = ("achieved counts the FP64-equivalent algorithmic flops; in the mixed form the "
                                   "step and Dyson run them as double-float on the FP32 pipe, so frac (of the "
                                   "FP64 pipe's measured peak) can exceed 1")
    if not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline(cfg, target_s=args.cpu_seconds)
        except Exception as e:  # reported, never silently substituted
            out["cpu_baseline"] = {"error": str(e)[:300]}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
