"""bench.py as the driver launches it for N > 1 (torchrun, one process per GPU, gloo for the timing
reduction), on CPU: the reference arm with two ranks prints exactly one JSON line (rank 0) and both
ranks exit 0; and the GPU arm's replica arithmetic (MAX of the ranks' frame times, vertex-steps of all
ranks together) on two gloo ranks."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks(oracle_lib):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--config", "small", "--gpus", "2", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def _aggregate_rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = [2.0, 3.5][rank]          # rank 1 is the slower replica
    q.put((rank, bench.replica_aggregate(ms_local, 1_000_000, world, dist)))
    dist.destroy_process_group()


def test_replica_aggregate_two_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_aggregate_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        ms, value = res[r]
        assert ms == 3.5                               # the slowest rank's time, on every rank
        assert abs(value - 2 * 1_000_000 / 3.5e-3) < 1e-6 * value   # both ranks' vertices per that time


def test_replica_aggregate_one_rank():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_aggregate(2.0, 500, 1) == (2.0, 500 / 2e-3)
