"""The N>1 path of bench.py on CPU: world_size-2 gloo process groups.

The GPU arm runs one replica per GPU (the path shards with no exchange);
its only cross-rank step is the max-over-ranks of the timed step and the
whole-job throughput built from it.  Those helpers are exercised here over
gloo, and the reference arm is launched under torchrun with two ranks
(rank 0 alone measures and prints; the other exits without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # per-rank step times: the job takes the slowest replica's
        mine = [0.1 * (rank + 1), 0.5 - 0.1 * rank, 0.25]
        got = bench.max_over_ranks(mine, world, "cpu")
        value = bench.job_throughput(world, 128, got[0])
        dist.barrier()
        q.put((rank, got, value))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value in res:
        assert got == pytest.approx([0.2, 0.5, 0.25])
        assert value == pytest.approx(2 * 128 / 0.2)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([0.3, 0.1], 1, "cpu") == [0.3, 0.1]
    assert bench.job_throughput(1, 48, 0.5) == pytest.approx(96.0)


def test_reference_arm_under_torchrun_two_ranks():
    """`bench.py --impl reference` launched by torch.distributed.run with two
    ranks: only rank 0 runs the CPU step and prints one JSON line."""
    oracle = pytest.importorskip("oracle")
    try:
        oracle.lib()
    except Exception as e:  # the C oracle is built by __graft_entry__.build()
        pytest.skip("oracle library not built: %s" % e)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c1",
           "--steps", "1", "--warmup", "0", "--gpus", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"

