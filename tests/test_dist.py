"""The N > 1 launch path on CPU (gloo, world size 2): bench.py's replicas share no data, only a
barrier and the max of the timings over ranks, and only rank 0 prints its JSON line."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(1.0 + rank)
    d.barrier()
    with open(out / f"r{rank}.txt", "w") as f:
        f.write(f"{d.rank} {d.world} {m}")
    d.td.destroy_process_group()


def test_dist_barrier_and_max_over_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, tmp_path)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        rank, world, m = (tmp_path / f"r{r}.txt").read_text().split()
        assert (int(rank), int(world), float(m)) == (r, 2, 2.0)


def test_reference_arm_two_ranks_prints_one_line():
    """torchrun with two ranks: rank 0 times the reference's CPU path and prints the line,
    rank 1 exits 0 without work."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_port()), str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cpu-seconds", "1", "--config", "c0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port")
    assert d["e2e"]["h2d_bytes_per_step"] == 0
