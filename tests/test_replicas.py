"""The multi-GPU path is replicas only (every pair is independent): bench.py under torchrun runs
one replica per rank, joined by a gloo barrier and a max-over-ranks of the step time.  These
CPU tests run that host logic with two gloo ranks on 127.0.0.1 (no GPU)."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2", LOCAL_RANK=str(rank))
    import bench
    d = bench.dist_init(2)
    v = bench.max_over_ranks(d, 1.5 + rank)
    d.barrier()
    out.put((rank, v))
    d.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_reference_arm_under_torchrun_prints_one_line():
    """`bench.py --impl reference` launched as the driver launches N > 1 runs: rank 0 times
    the CPU restatement and prints the line, the other rank exits 0 without work."""
    pytest.importorskip("torch.distributed.run")
    build = subprocess.run([sys.executable, "-c", "import oracle.build as b; b.build()"],
                           cwd=ROOT, capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--config", "c1", "--scale", "0.005", "--ref-seconds", "0.2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
    assert lines[0]["value"] > 0 and lines[0]["cpu_baseline"]["kind"] == "port"
