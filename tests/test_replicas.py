"""The multi-GPU mode's host logic (generic-linalg_gb300/replicas.py) on CPU ranks: systems are
shared out with no overlap and balanced cost, each rank solves its share (here with the oracle's
FP64 CG, standing in for the device solve), the per-system results are gathered, and the job
time is the slowest rank's.  world_size 2 over gloo on 127.0.0.1."""
from __future__ import annotations

import importlib
import importlib.util
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _replicas():
    """replicas.py on its own (pure host logic: it needs neither the CUDA library nor a GPU)."""
    spec = importlib.util.spec_from_file_location("glinalg_replicas",
                                                  os.path.join(ROOT, "generic-linalg_gb300", "replicas.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_shard_covers_every_system_once_and_balances():
    rep = _replicas()
    rng = np.random.default_rng(0)
    costs = [float(s * s) for s in rng.choice([32, 64, 128, 256], size=256)]
    for world in (1, 2, 3, 8):
        shares = rep.shard_by_cost(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shares]
        # greedy largest-first: no rank exceeds the mean by more than the largest single cost
        assert max(loads) - sum(loads) / world <= max(costs)
    assert rep.shard_by_cost([], 2) == [[], []]
    assert rep.shard_by_cost([5.0], 2) == [[0], []]
    with pytest.raises(ValueError):
        rep.shard_by_cost([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _systems():
    """Six small staggered systems (sides 8..16) from a seeded numpy generator."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    ref = pyoracle.Oracle()
    rng = np.random.default_rng(1)
    out = []
    for q in range(6):
        L = int(rng.choice([8, 12, 16]))
        U = np.exp(1j * rng.uniform(-np.pi, np.pi, 2 * L * L))
        b = rng.normal(size=L * L) + 1j * rng.normal(size=L * L)
        out.append((L, 0.1 + 0.05 * q, U, b))
    return ref, pyoracle, out


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rep = _replicas()
        ref, pyoracle, systems = _systems()
        costs = [L * L for L, *_ in systems]
        local = {}
        for i in rep.my_share(costs, rank, world):
            L, m, U, b = systems[i]
            op = pyoracle.Operator("staggered_normal", L, L, m, U)
            x, info, _ = ref.solve("cg", op, b, max_iter=10000, eps=1e-10)
            local[i] = (info["iter"], x)
        allres = rep.gather_results(local, world)
        t = rep.max_over_ranks(float(rank + 1), world)
        if rank == 0:
            np.savez(os.path.join(outdir, "gathered.npz"),
                     idx=np.array(sorted(allres)), iters=np.array([allres[i][0] for i in sorted(allres)]),
                     t=np.array([t]), **{f"x{i}": allres[i][1] for i in allres})
    finally:
        dist.destroy_process_group()


def test_two_ranks_solve_their_shares_and_gather(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = np.load(tmp_path / "gathered.npz")
    assert list(got["idx"]) == list(range(6))
    assert got["t"][0] == 2.0  # the slower rank's time
    ref, pyoracle, systems = _systems()
    for i, (L, m, U, b) in enumerate(systems):
        op = pyoracle.Operator("staggered_normal", L, L, m, U)
        x, info, _ = ref.solve("cg", op, b, max_iter=10000, eps=1e-10)
        assert got["iters"][i] == info["iter"]
        assert np.array_equal(got[f"x{i}"], x)


def test_gather_rejects_a_system_solved_twice(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    with pytest.raises(Exception):
        mp.start_processes(_dup_main, args=(2, port), nprocs=2, join=True, start_method="spawn")


def _dup_main(rank, world, port):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _replicas().gather_results({0: rank}, world)  # both ranks claim system 0
    finally:
        dist.destroy_process_group()
