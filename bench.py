#!/usr/bin/env python3
"""Benchmark: powder FIDs/s of the spinning powder-FID path on one GB300, mixed precision
against plain FP64.

A step is one powder-averaged FID of the workload.  Default: c2 (8 x 1H, dim 256, 1154 ZCW
crystallites, 200 steps per rotor period, 4096 points; blochlib_gb300/workloads.py) in the
mixed form, with the FP64 form of the same job beside it, and the other configurations as
extra keys of the same line: c1 (both forms), c3 (the batching form: 512 seeded systems
through the serving loop, both forms) and c4 (the serving form: a 60 s Poisson stream, both
forms, p50/p99).

  value     FIDs/s of the mixed form with every input resident in HBM (bl_job_run), CUDA
            events on the engine's stream around exactly K steps, max over ranks.
  precision_forms  the FP64 form of the same job, the mixed form's relative L2 error against
            it and the speed-up.
  e2e       FIDs/s through the reference-facing call (oneFID.FID -> bl_powder_fid: host buffers
            in, upload, compute, FID read back), wall clock around the calls.
  roofline  per stage: algorithmic flop per run / CUDA-event time per run against the unit
            that bounds the stage (FP64 pipe: live DFMA probe; FP32 pipe: live FFMA probe;
            tensor pipe: MEASURED_PEAKS.json bf16); the headline is the stage with the largest
            share of the timed region.
  cpu_baseline  the reference's own CPU path (oracle/_ref/ref_fid, as shipped), one process
            per host core on a bounded crystallite sample, scaled to FIDs/s; the CPU
            restatement (oracle) where the reference binary is absent.

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
# the mixed form's arithmetic (blocks up to 8: double-float step and Dyson; 9-39: the same on CTA-wide kernels;
# 40-74: exact-slice BF16 products on the tensor cores)
MIXED_DTYPE = ("bf16 tensor-core exact slices (step, Dyson, blocks 40-74) + df32 double-float (smaller blocks' step "
               "and Dyson; Floquet Cayley, V, eigenvalues) + f32 (Floquet sweeps, eigenframe, Q/R, Fave, FID) + "
               "f64 (powder sum)")


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
    """One process per core, each on its own contiguous crystallite range of k crystallites:
    first k = 1 (one crystallite per core already exceeds target_s for c2), then, if that
    took well under target_s, k scaled up to fill it.  Returns FIDs/s scaled from the sample."""
    binary, kind = _ref_binary()
    cores = cores or os.cpu_count() or 1
    C = len(cfg["powder"][0])
    with tempfile.TemporaryDirectory() as tmp:
        k = 1
        ranges = [(i * max(1, C // cores) % max(C - k + 1, 1), k) for i in range(cores)]
        wall = _cpu_run(binary, cfg, ranges, tmp)
        if wall < 0.4 * target_s:
            k = int(max(1, min(max(1, C // cores), round(target_s / max(wall, 1e-4)))))
            if k > 1:
                ranges = [(i * k % max(C - k + 1, 1), k) for i in range(cores)]
                wall = _cpu_run(binary, cfg, ranges, tmp)
    fids = cores * k / C
    return {"value": fids / wall, "unit": UNIT, "cores": cores, "kind": kind, "wall_s": wall,
            "sample": f"{cores} processes x {k} crystallite(s) ({cores * k} of {C}) of the full workload, "
                      f"{wall:.1f} s wall, extrapolated linearly to the whole powder (FIDs/s)",
            "binary": str(binary.relative_to(ROOT))}


def workload_name(cfg):
    """The workload string both arms print (the precision form goes in its own config key)."""
    dim = 2 ** int(cfg["lines"][0].split()[1]) if cfg["lines"][0].startswith("numspin") else 0
    spins = [l.split()[1] for l in cfg["lines"] if l.startswith("T ")]
    kinds = sorted(set(spins))
    desc = " + ".join(f"{spins.count(x)} x {x}" for x in kinds)
    return (f"{cfg['name']}: {desc} (dim {dim}), {len(cfg['powder'][0])} crystallites, "
            f"{describe(cfg, dim)}, npts={cfg['npts']}")


# ------------------------------------------------------------------ main
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cfg = workload(args)
    if args.crystallites:
        cfg = dict(cfg, powder=tuple(np.asarray(x)[:args.crystallites] for x in cfg["powder"]))
    binary, kind = _ref_binary()
    from blochlib_gb300 import workloads as W
    small = W.config(0)
    small = dict(small, powder=tuple(np.asarray(x)[:1] for x in small["powder"]))
    for _ in range(args.warmup):  # pages the binary in; the CPU path has no device to warm
        cpu_baseline(small, target_s=0.0, cores=1)
    vals, walls = [], []
    for _ in range(args.steps):
        r = cpu_baseline(cfg, target_s=args.cpu_seconds)
        vals.append(r["value"])
        walls.append(r["wall_s"])
    v = statistics.median(vals)
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(walls),
           "ms_per_fid_extrapolated": 1e3 / v, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, workloads.py)",
           "config": {"workload": workload_name(cfg), "precision": "fp64 (the reference's CPU path)"},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["cores"], "kind": kind,
                            "sample": "per step: " + r["sample"]},
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


def batch_form(args, local, systems):
    """c3: seeded spin systems (2..7 1H, n 64..256, 1024 points, powders of 144..1154)
    submitted at once to the serving loop; FIDs/s of the whole batch, mixed and FP64."""
    import blochlib_gb300 as bl
    from blochlib_gb300 import workloads as W
    cfgs = [W.config(3, i) for i in range(systems)]
    jobs = [_job_inputs(bl, c) for c in cfgs]
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
    errs = [_rel(a, b) for a, b in zip(fids["mixed"], fids["fp64"]) if a is not None and b is not None]
    forms["mixed"]["rel_err_vs_fp64_max"] = max(errs) if errs else None
    forms["mixed_speedup_vs_fp64"] = forms["mixed"]["fids_per_s"] / forms["fp64"]["fids_per_s"]
    dims = sorted({2 ** int(c["lines"][0].split()[1]) for c in cfgs})
    forms["workload"] = (f"c3 batching form: {len(cfgs)} seeded systems, dims {dims}, n 64-256, 1024 points, "
                         "powders 144/320/678/1154, all submitted at once")
    forms["lanes"] = args.lanes
    return forms


def run_batch(args):
    rank, world, local = dist_env()
    import blochlib_gb300 as bl
    peak = bl.probe_fp64_tflops(bl.Context(local))
    clocks = Clocks(local)
    clocks.start()
    forms = batch_form(args, local, args.systems)
    clk = clocks.stop()
    if rank != 0:
        return 0
    print(json.dumps({
        "metric": METRIC, "value": forms["mixed"]["fids_per_s"], "unit": UNIT, "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": 1e3 * forms["mixed"]["seconds"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": MIXED_DTYPE, "data": "synthetic (seeded, workloads.py config 3)",
        "config": {"workload": forms["workload"], "lanes": args.lanes, "pool_gib": args.pool_gib,
                   "precision": "mixed (FP64 row for comparison)"},
        "latency_ms": forms["mixed"]["latency_ms"], "precision_forms": forms,
        "roofline": {"bound": "fp64", "kernel": "whole batch (all stages)", "form": "fp64",
                     "achieved": forms["fp64"]["tflops_algorithmic"], "peak": peak, "unit": "TFLOP/s",
                     "frac": forms["fp64"]["tflops_algorithmic"] / peak if peak else None, "traffic": None,
                     "peak_source": "measured live: DFMA probe kernel"},
        "clocks": clk}))
    return 0


def serving_form(args, local, duration):
    """c4: Poisson request stream (seeded) of c3-like jobs plus 10% large jobs (9-10 x 1H,
    dims 512-1024, on the 100-point repulsion set), for a fixed window; the backlog left at
    the end is cancelled and reported.  Mixed and FP64 on the same stream."""
    import blochlib_gb300 as bl
    from blochlib_gb300 import workloads as W
    rng = np.random.default_rng(W.SEED0 + 4)
    small = [_job_inputs(bl, W.config(3, 1000 + i)) for i in range(48)]
    large = [_job_inputs(bl, W.config(4, i)) for i in range(4)]
    n_req = int(args.rate * duration)
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
                       "finished_after_drain": sum(v[0] == srv.DONE for v in late.values()),
                       "achieved_fids_per_s": len(ok) / total, "window_s": window, "total_s": total,
                       "latency_ms": {"p50": float(np.percentile(ok, 50)) if ok else None,
                                      "p99": float(np.percentile(ok, 99)) if ok else None}}
        srv.close()
    forms["mixed_speedup_vs_fp64"] = forms["mixed"]["achieved_fids_per_s"] / forms["fp64"]["achieved_fids_per_s"]
    forms["workload"] = (f"c4 serving form: Poisson {args.rate:g}/s for {duration:g} s, 90% c3-like, 10% 9-10 x 1H "
                         "(dims 512-1024) on rep100")
    forms["lanes"] = args.lanes
    forms["drain_s"] = args.drain
    return forms


def run_serving(args):
    rank, world, local = dist_env()
    forms = serving_form(args, local, args.duration)
    if rank != 0:
        return 0
    print(json.dumps({
        "metric": METRIC, "value": forms["mixed"]["achieved_fids_per_s"], "unit": UNIT, "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": 1e3 * forms["mixed"]["total_s"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": MIXED_DTYPE, "data": "synthetic seeded Poisson stream (workloads.py)",
        "config": {"workload": forms["workload"], "lanes": args.lanes, "pool_gib": args.pool_gib,
                   "drain_s": args.drain},
        "latency_ms": forms["mixed"]["latency_ms"], "precision_forms": forms}))
    return 0


# stage -> (pipe of the FP64 form, pipe of the mixed form); in the mixed form the step and Dyson of
# blocks of 40-74 run on the tensor cores (their stages are reported as "tensor" when the kernels
# counted tensor flops), smaller blocks and the Floquet step in double-float on the FP32 pipe
STAGE_PIPE = {"k_step_prop": ("fp64", "fp32"), "k_dyson": ("fp64", "fp32"), "k_floquet": ("fp64", "fp32"),
              "k_eigframe": ("fp64", "fp32"), "k_qr": ("fp64", "fp32"), "k_fave": ("fp64", "fp32"),
              "k_fid": ("fp64", "fp32"), "k_reduce": ("fp64", "fp64")}


def measured_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return json.loads(f.read_text())
    except (OSError, ValueError):
        return {}


def measure_job(args, d, ctx, cfg, prec, steps, warmup, compare, e2e_steps, peaks):
    """One workload as a single resident job: the timed form `prec`, the other form for the
    error and the speed-up, and the e2e call.  Returns the fields of the JSON line."""
    import blochlib_gb300 as bl
    s, pw, ro, det, job = make_job(bl, cfg, ctx, args.step_method, args.fave_method, 1 if prec == "mixed" else 0)
    for _ in range(warmup):
        job.run()
    job.sync()
    clocks = Clocks(d.local)
    clocks.start()
    time.sleep(0.5)
    job.set_profiling(True)
    job.reset_stage_times()
    d.barrier()
    job.sync()
    per_step = [job.run_timed(1) for _ in range(steps)]
    job.sync()
    d.barrier()
    ms_total = sum(per_step)
    clk = clocks.stop()
    ms_max = d.max(ms_total)
    value = d.world * steps / (ms_max / 1e3)
    fid_main = job.read()
    stages = job.stage_times()
    sflops = job.stage_flops()
    if "p2p" in cfg:  # stage 5 runs the point-to-point terms instead of the Fave correlation
        stages = {("k_p2p_elems" if k == "k_fave" else k): v for k, v in stages.items()}
        sflops = {("k_p2p_elems" if k == "k_fave" else k): v for k, v in sflops.items()}
    layout = job.describe()
    tf_step, tf_dyson = job.tensor_flops() if prec == "mixed" else (0.0, 0.0)
    launches_per_run = job.launches
    job.set_profiling(False)
    # per-stage roofline against the unit that bounds the stage
    col = 1 if prec == "mixed" else 0
    per_stage = {}
    for k, (ms, nl) in stages.items():
        if ms <= 0:
            continue
        t = ms / steps / 1e3
        pipe = STAGE_PIPE.get(k, ("fp64", "fp32"))[col]
        tfl = {"k_step_prop": tf_step, "k_dyson": tf_dyson}.get(k, 0.0)
        if tfl > 0:
            pipe = "tensor"
        elif pipe == "tensor":
            pipe = "fp32"  # no tensor-core block in this job: double-float on the FP32 pipe
        e = {"share": ms / ms_total, "ms_per_run": ms / steps, "launches_per_run": nl / steps, "pipe": pipe,
             "algorithmic_tflops_fp64_equiv": sflops.get(k, 0.0) / t / 1e12}
        if pipe == "fp64":
            e.update(peak=peaks["fp64"], frac=e["algorithmic_tflops_fp64_equiv"] / peaks["fp64"])
        elif pipe == "tensor":
            tf = tfl / t / 1e12
            e.update(bf16_tflops_issued=tf, peak=peaks["bf16"], frac=tf / peaks["bf16"],
                     note="BF16 flops of the exact-slice products (counted by the kernels) over the stage's "
                          "CUDA-event time, which also covers the stage's double-float small-block kernels")
        else:  # single precision: the algorithmic count is the FP32 count (double-float stages issue ~12x more)
            e.update(peak=peaks["fp32"], frac=e["algorithmic_tflops_fp64_equiv"] / peaks["fp32"])
        per_stage[k] = e
    dom = max(per_stage, key=lambda k: per_stage[k]["share"])
    D = per_stage[dom]
    if D["pipe"] == "tensor":
        roof = {"bound": "tensor", "achieved": D["bf16_tflops_issued"], "peak": peaks["bf16"], "unit": "TFLOP/s",
                "frac": D["frac"], "peak_source": peaks["bf16_source"],
                "algorithmic_unit": "BF16 flops of the exact-slice products: 10 slice pairs x 2 b^3 per real "
                                    "b x b product (unpadded), counted by the tensor-core kernels"}
    elif D["pipe"] == "fp32":
        ach = D["algorithmic_tflops_fp64_equiv"]
        roof = {"bound": "fp32", "achieved": ach, "peak": peaks["fp64"], "unit": "TFLOP/s (FP64-equivalent)",
                "frac": ach / peaks["fp64"], "fp32_pipe_peak": peaks["fp32"],
                "peak_source": "measured live: DFMA probe kernel (frac = FP64-equivalent work over the FP64 "
                               "pipe's peak; the stage runs it as double-float on the FP32 pipe, FFMA probe "
                               "peak beside it)"}
    else:
        ach = D["algorithmic_tflops_fp64_equiv"]
        roof = {"bound": "fp64", "achieved": ach, "peak": peaks["fp64"], "unit": "TFLOP/s", "frac": ach / peaks["fp64"],
                "peak_source": "measured live: DFMA probe kernel (MEASURED_PEAKS.json has no FP64 figure)"}
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(cfg["name"], {}).get(prec, {}).get(dom)
        except (ValueError, AttributeError):
            traffic = None
    roof.update(kernel=dom, form=prec, traffic=traffic, stages=per_stage)
    forms = {prec: {"fids_per_s": value, "ms_per_fid": ms_max / steps}}
    if compare:
        other = "fp64" if prec == "mixed" else "mixed"
        _, _, _, _, job2 = make_job(bl, cfg, ctx, args.step_method, args.fave_method, 1 if other == "mixed" else 0)
        job2.run()
        job2.sync()
        k2 = max(1, min(steps, args.compare_steps))
        ms2 = job2.run_timed(k2) / k2
        fid_other = job2.read()
        forms[other] = {"fids_per_s": 1e3 / ms2, "ms_per_fid": ms2, "timed_steps": k2, "warmup": 1}
        f64, fmx = (fid_main, fid_other) if prec == "fp64" else (fid_other, fid_main)
        forms["mixed"]["rel_err_vs_fp64"] = _rel(fmx, f64)
        forms["mixed_speedup_vs_fp64"] = forms["mixed"]["fids_per_s"] / forms["fp64"]["fids_per_s"]
        job2.close()
    # e2e through the reference-facing call with host buffers, the resident job closed first so
    # that the call sees the device as a caller's would (its batches sized from the free memory)
    h2d, d2h = job.io_bytes()
    h2d += 8 * 4 * len(cfg["powder"][0]) + 2 * ro.nbytes  # the caller's powder arrays and rho/det
    job.close()
    drv = bl.oneFID(s, cfg["npts"], cfg["sw"], cfg["wr"], cfg["rotb"], ctx=ctx, step_method=args.step_method,
                    fave_method=args.fave_method, precision=1 if prec == "mixed" else 0)
    drive_fid(bl, cfg, drv, pw, ro, det)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        drive_fid(bl, cfg, drv, pw, ro, det)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    return {"value": value, "ms_per_step": ms_max / steps, "per_step": per_step, "forms": forms, "roofline": roof,
            "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": e2e_steps, "call": "oneFID.FID -> bl_powder_fid"},
            "gpu_launches": launches_per_run * steps, "clocks": clk, "layout": layout, "dim": s.dim()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c0", "c1", "c2", "c3", "c4"])
    ap.add_argument("--systems", type=int, default=512, help="c3: number of seeded systems in the batch")
    ap.add_argument("--system", type=int, default=None,
                    help="c3/c4: time this one seeded system as a single job instead of the batching/serving form")
    ap.add_argument("--period-steps", type=int, default=0, help="override the steps per rotor period (sw = n wr)")
    ap.add_argument("--lanes", type=int, default=16, help="c3/c4: serving lanes (CUDA streams)")
    ap.add_argument("--pool-gib", type=int, default=128, help="c3/c4: serving memory pool (GiB)")
    ap.add_argument("--rate", type=float, default=200.0, help="c4: offered requests per second")
    ap.add_argument("--duration", type=float, default=60.0, help="c4: arrival window (s)")
    ap.add_argument("--drain", type=float, default=20.0, help="c4: wait after the window (s)")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--compare-steps", type=int, default=2, help="timed runs of the other precision form")
    ap.add_argument("--p2p", type=int, nargs=2, default=None, metavar=("BASE", "FACTOR"),
                    help="point-to-point FID every FACTOR/BASE rotor periods instead of gamma-COMPUTE")
    ap.add_argument("--maxtstep", type=float, default=0.0, help="--p2p: longest step inside a chunk (s)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default c2 run: skip the c1, c3 (batching) and c4 (serving) keys")
    ap.add_argument("--crystallites", type=int, default=0,
                    help="use only the first N crystallites (smaller case for profiler captures)")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"],
                    help="path timed for 'value' (default: mixed for c2, fp64 for c0/c1)")
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
    mp = measured_peaks()
    peaks = {"fp64": bl.probe_fp64_tflops(ctx), "fp32": bl.probe_fp32_tflops(ctx),
             "bf16": mp.get("bf16_tflops_sustained") or 1700.0,
             "bf16_source": ("MEASURED_PEAKS.json bf16_tflops_sustained (kernel inside a long step)"
                             if mp.get("bf16_tflops_sustained") else "fallback 1.7 PFLOP/s sustained")}
    r = measure_job(args, d, ctx, cfg, prec, args.steps, args.warmup, not args.no_compare, args.e2e_steps, peaks)
    extras = {}
    if (args.config == "c2" and not args.no_extras and not args.crystallites and not args.period_steps
            and not args.p2p):
        c1 = workload(argparse.Namespace(config="c1", system=None, period_steps=0, p2p=None, maxtstep=0.0))
        r1 = measure_job(args, d, ctx, c1, "mixed", 5, 3, True, 2, peaks)
        extras["c1"] = {"workload": workload_name(c1), "precision_forms": r1["forms"],
                        "e2e_mixed": r1["e2e"]["value"],
                        "roofline_dominant": {k: r1["roofline"][k] for k in ("kernel", "bound", "frac")}}
        extras["c3_batching"] = batch_form(args, d.local, args.systems)
        extras["c4_serving"] = serving_form(args, d.local, args.duration)
    if d.rank != 0:
        return 0
    dtype = "f64" if prec == "fp64" else MIXED_DTYPE
    out = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": d.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded spin systems and ZCW powder, workloads.py)",
        "config": {"workload": workload_name(cfg), "precision": prec, "step_method": args.step_method,
                   "parallelism": f"replicas x{d.world}",
                   "l2": "inputs larger than L2: each step streams the per-crystallite work buffers (GBs)",
                   "layout": r["layout"]},
        "latency_ms": {"p50": float(np.percentile(r["per_step"], 50)), "p99": float(np.percentile(r["per_step"], 99))},
        "precision_forms": r["forms"],
        "roofline": r["roofline"],
        "e2e": r["e2e"],
        "gpu_launches": r["gpu_launches"],
        "clocks": r["clocks"],
        "peaks": {k: v for k, v in peaks.items()},
    }
    out.update(extras)
    if not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline(cfg, target_s=args.cpu_seconds)
        except Exception as e:  # reported, never silently substituted
            out["cpu_baseline"] = {"error": str(e)[:300]}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
