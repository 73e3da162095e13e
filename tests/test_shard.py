"""Sharding of independent problems over ranks (CPU, gloo, world size 2): the
partition is complete and balanced, and the gathered results come back in the
original order, equal to solving everything on one rank."""
import os
import socket

import numpy as np
import pytest

from gplite_gb300.shard import balance, partition, solve_sharded


def test_partition_complete_and_balanced():
    rng = np.random.default_rng(0)
    sizes = [int(np.exp(rng.uniform(np.log(64), np.log(1024)))) for _ in range(4096)]
    for world in (1, 2, 4, 8):
        parts = partition(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        assert balance(parts, sizes) < 1.01
    assert partition(sizes, 4) == partition(sizes, 4)  # deterministic


def oracle_solve(problems):
    from oracle import gplite_ref as R
    out = []
    for p in problems:
        gp = R.gp_init([R.cf("sexp", lscale=p["lscale"], magn=1.0)], R.lik("gaussian", sigma=p["sigma"]))
        out.append(float(R.gp_fit(gp, p["x"], p["y"]).fit["log_evidence"]))
    return out


def make(count=12, seed=2):
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(count):
        n = int(rng.integers(5, 60))
        x = rng.uniform(-2, 2, (n, 1))
        probs.append(dict(x=x, y=np.sin(2 * x[:, 0]) + 0.1 * rng.standard_normal(n), lscale=0.5, sigma=0.2))
    return probs


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = solve_sharded(make(), oracle_solve)
        q.put((rank, res))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_results_match_single_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = oracle_solve(make())
    for r in (0, 1):
        assert got[r] == pytest.approx(ref, rel=0, abs=0)
