"""The multi-rank (replica) logic of bench.py on CPU with the gloo backend,
world size 2: the timed region is the slowest rank's, every rank draws its
own walkers, and the reference arm prints exactly one line (rank 0)."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank)
    q.put((rank, ms, bench.walker_seed(100, rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_walker_seeds():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]  # both ranks see the slowest time
    assert out[0][2] != out[1][2]  # distinct walkers per rank
    sys.path.insert(0, os.path.join(ROOT, "cocoa-cosmolike-core_gb300"))
    from cl2pt import workloads
    w = workloads.make("real_3x2pt_small")
    t0, _ = workloads.points(w, 2, seed=out[0][2])
    t1, _ = workloads.points(w, 2, seed=out[1][2])
    assert not np.array_equal(t0[0].lnP, t1[0].lnP)


def test_reference_arm_prints_once_on_rank0():
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "real_3x2pt_small", "--steps", "1", "--warmup", "0",
           "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
