"""N > 1 paths, on CPU.

bench.py --gpus N runs one independent replica per rank (the path has no
cross-GPU exchange); the job time is the max over ranks.  That reduction and
the reference arm's rank handling are exercised here with world_size-2 gloo
process groups (127.0.0.1 rendezvous), no GPU."""
import json
import os
import socket
import subprocess
import sys

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.reduce_max(10.0 + rank * 5.0, world)
    units = torch.tensor([16.0])
    dist.all_reduce(units)  # every replica solves its own 16-RHS block
    q.put((rank, t, float(units.item())))
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert [r[2] for r in res] == [32.0, 32.0]


def test_reference_arm_json_and_nonzero_ranks():
    env = dict(os.environ)
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload",
                          "st27_32_m16", "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    line = [l for l in out.stdout.splitlines() if l.startswith("{")][-1]
    d = json.loads(line)
    assert d["impl"] == "reference"
    if "unavailable" not in d:
        assert d["value"] > 0 and d["unit"] == "RHS/s"
        assert d["cpu_baseline"]["kind"] == "reference" and d["cpu_baseline"]["cores"] >= 1
        assert d["e2e"]["h2d_bytes_per_step"] == 0
    env.update(RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload",
                          "st27_32_m16", "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip() == ""
