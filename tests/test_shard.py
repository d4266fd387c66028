"""Sharded batches on several ranks (host logic, gloo on CPU) and the seeded workloads.

A batch shards by whole tests (independent units, no data-path collective); ranks
gather (index, Res64, status, round-off) records once at the end.  Here two gloo ranks
on 127.0.0.1 run the sharded path with the exact CPU oracle standing in for the GPU
runner, and rank 0's merged result must equal a single-process run.
"""
import os
import socket

import numpy as np
import pytest

from gpulucas_gb300 import shard, workloads


def test_partition_balances_and_covers():
    rng = np.random.default_rng(0)
    costs = list(rng.uniform(1, 100, 257))
    for world in (1, 2, 3, 8):
        parts = shard.partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs) + 1e-9


def test_batch_exponents_deterministic():
    a = workloads.batch_exponents()
    b = workloads.batch_exponents()
    assert a == b and len(a) == 256 and len(set(a)) == 256
    assert all(100_000 <= p <= 3_000_000 and workloads.is_prime(p) for p in a)
    assert workloads.batch_exponents(seed=5) != a


def test_primality_helpers():
    sympy = pytest.importorskip("sympy")
    for n in list(range(0, 2000)) + [2976221, 43112609, 43112611, 1000003, 999999937, 2**31 - 1]:
        assert workloads.is_prime(n) == bool(sympy.isprime(n)), n
    ps = workloads.primes_between(100, 5000)
    assert list(ps) == list(sympy.primerange(100, 5001))


def test_serving_requests_shape():
    reqs = workloads.serving_requests(400)
    t = [r.arrival_s for r in reqs]
    assert all(b > a for a, b in zip(t, t[1:]))
    assert 4.0 < t[-1] < 12.0                      # mean rate 50/s
    full = [r for r in reqs if r.full]
    assert 0.1 < len(full) / len(reqs) < 0.3
    assert all(r.iterations == r.p - 2 and r.p < 2_000_100 for r in full)
    assert all(r.iterations == 5000 for r in reqs if not r.full)
    assert all(workloads.is_prime(r.p) and 100_000 <= r.p <= 50_000_100 for r in reqs)


def _oracle_runner(ps, Ns, iterations, device=0):
    import oracle
    return [(oracle.Exact(p).iterate(iterations).res64(), 0, 0.0) for p in ps]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, ps, Ns, iters, out_path):
    import pickle
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from gpulucas_gb300 import shard as sh
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)

    def gather(obj):
        parts = [None] * world
        dist.all_gather_object(parts, obj)
        return parts

    devices = []

    def runner(ps_, Ns_, it, device):
        devices.append(device)
        return _oracle_runner(ps_, Ns_, it, device)

    os.environ["LOCAL_RANK"] = str(rank)
    res = sh.run_sharded(ps, Ns, iters, rank, world, runner, gather)
    seen = gather(devices)
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        with open(out_path, "wb") as f:
            pickle.dump((res, seen), f)


def test_sharded_run_two_gloo_ranks(tmp_path):
    import pickle

    import torch.multiprocessing as mp
    ps = [521, 607, 1279, 2203, 2281, 3217, 4253, 4423, 521, 9689]
    Ns = [32, 32, 64, 128, 128, 160, 256, 256, 32, 512]
    iters = 60
    out = str(tmp_path / "res.pkl")
    mp.start_processes(_rank_main, args=(2, _free_port(), ps, Ns, iters, out), nprocs=2, join=True,
                       start_method="spawn")
    with open(out, "rb") as f:
        res, seen = pickle.load(f)
    assert res == _oracle_runner(ps, Ns, iters)
    # each rank ran its share on its own device (LOCAL_RANK), not all on device 0
    assert seen == [[0], [1]]


def test_local_device(monkeypatch):
    monkeypatch.delenv("LOCAL_RANK", raising=False)
    assert shard.local_device(3) == 3 and shard.local_device(9, 8) == 1
    monkeypatch.setenv("LOCAL_RANK", "5")
    assert shard.local_device(13) == 5 and shard.local_device(13, 4) == 1


@pytest.mark.gpu
def test_sharded_gpu_runner_one_rank_matches_golden(gl):
    """run_sharded with the GPU runner on this process's GPU (world 1, no gather): the
    batched configuration's golden exponents after 10000 iterations."""
    import json
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "res64_batch.json")) as f:
        golden = json.load(f)
    ps = [e["p"] for e in golden]
    Ns = [e["N"] for e in golden]
    recs = shard.run_sharded(ps, Ns, 10000, 0, 1, shard.gpu_runner, device=0)
    assert [r[0] for r in recs] == list(range(len(ps)))
    for (i, res64, st, err), e in zip(recs, golden):
        assert st == 0 and err < 0.4
        assert f"{res64:016x}" == e["res64"], e["p"]
