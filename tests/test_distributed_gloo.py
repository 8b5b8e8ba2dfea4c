"""The benchmark's multi-rank path on CPU (gloo, world size 2).

Multi-GPU runs of this path are replicas: each rank factors its own matrix and
the only cross-rank operations are the timing barrier and a MAX reduction of
the elapsed time.  Those helpers are checked here with two gloo ranks, and the
reference arm is launched as a multi-GPU bench run launches it (torchrun, 2 ranks):
rank 0 prints the one JSON line, rank 1 exits 0 without work.
"""
import json
import multiprocessing as mp
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


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    v = bench.reduce_max(1.5 * (rank + 1), world)    # ranks time 1.5 ms and 3.0 ms
    bench.barrier(world)
    q.put((rank, v))
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(out) == [(0, 3.0), (1, 3.0)]


def test_reference_arm_under_torchrun_two_ranks(tmp_path):
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                            # rank 0 only
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import numpy as np
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, os.path.join(ROOT, "nextla.jl_gb300"))
    from tileqr import batched as Bt
    ms, ns, ks = Bt.random_sizes(4096, seed=7)
    mine = Bt.shard(ms, ns, ks, world, rank)
    # each rank "solves" its problems (a per-problem value standing in for X)
    vals = torch.tensor([float(ms[i] * 7 + ns[i]) for i in mine], dtype=torch.float64)
    idx = torch.tensor(mine, dtype=torch.int64)
    # host-side gather of the results: the only cross-rank step
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([idx.numel()]))
    n_max = int(max(s.item() for s in sizes))
    pad_i = torch.full((n_max,), -1, dtype=torch.int64)
    pad_v = torch.zeros(n_max, dtype=torch.float64)
    pad_i[:idx.numel()] = idx
    pad_v[:vals.numel()] = vals
    gi = [torch.empty(n_max, dtype=torch.int64) for _ in range(world)]
    gv = [torch.empty(n_max, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gi, pad_i)
    dist.all_gather(gv, pad_v)
    cost = Bt.problem_cost(ms, ns, ks)
    q.put((rank, [g.tolist() for g in gi], [g.tolist() for g in gv], float(cost[mine].sum()), float(cost.sum())))
    dist.destroy_process_group()


def test_batched_shard_by_cost_gloo():
    """The batched solver and the differentiable QR shard by problem: each of two gloo ranks computes its
    part of the cost-balanced partition on its own, the parts cover the batch
    exactly once with costs within 0.1 % of each other, and a host-side gather
    puts every problem's result back in place."""
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    _, gi, gv, c0, total = out[0]
    _, gi1, gv1, c1, _ = out[1]
    assert gi == gi1 and gv == gv1                  # both ranks gathered the same
    seen = {}
    for r in range(2):
        for i, v in zip(gi[r], gv[r]):
            if i >= 0:
                assert i not in seen
                seen[i] = v
    assert sorted(seen) == list(range(4096))
    sys.path.insert(0, os.path.join(ROOT, "nextla.jl_gb300"))
    from tileqr import batched as Bt
    ms, ns, ks = Bt.random_sizes(4096, seed=7)
    assert all(seen[i] == float(ms[i] * 7 + ns[i]) for i in range(4096))
    assert abs(c0 - c1) / total < 1e-3
    assert abs(c0 + c1 - total) / total < 1e-12
    # one rank owns everything; the split is deterministic
    assert np.array_equal(Bt.shard(ms, ns, ks, 1, 0), np.arange(4096))
    assert np.array_equal(Bt.shard(ms, ns, ks, 3, 1), Bt.shard(ms, ns, ks, 3, 1))
