"""Sharding batched Lucas-Lehmer tests across GPUs (one process per GPU).

Tests are independent, so a batch shards by whole tests with no collective on the data
path: each rank takes the tests `partition` assigns it (greedy longest-processing-time
on the modelled FP64 work, FLOP_alg(N) x iterations), advances them in its own
gl_batch, and the host gathers (index, Res64, round-off) records at the end with one
all_gather_object.  The reference is single-process; this has no counterpart there.
"""
from __future__ import annotations

import heapq
import math
import os
from typing import Callable, Sequence


def flop_alg(N: int) -> float:
    """5 N log2 N + 4 N: real forward + inverse FFT, square, weight, unweight."""
    return 5.0 * N * math.log2(N) + 4.0 * N


def partition(costs: Sequence[float], world: int) -> list[list[int]]:
    """Indices of `costs` split over `world` ranks, largest first onto the least
    loaded rank; each rank's list is sorted.  Deterministic for equal costs."""
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(x) for x in out]


def local_device(rank: int, device_count: int | None = None) -> int:
    """The GPU of this rank on its node: LOCAL_RANK when the launcher sets it (torchrun
    does), else the global rank; modulo the visible device count when it is known."""
    dev = int(os.environ.get("LOCAL_RANK", rank))
    if device_count:
        dev %= device_count
    return dev


def run_sharded(ps: Sequence[int], Ns: Sequence[int], iterations: int, rank: int, world: int,
                runner: Callable[[list[int], list[int], int, int], list[tuple[int, int, float]]],
                gather: Callable[[object], list[object]] | None = None,
                device: int | None = None) -> list[tuple[int, int, float]] | None:
    """Run this rank's share on `device` (default: local_device(rank));
    `runner(ps, Ns, iterations, device)` returns one (res64, status, max_roundoff) per
    test.  With `gather` (an all_gather_object), rank 0 returns the records of all tests
    in input order, others None; without it, this rank's own (index, res64, status,
    max_roundoff) records."""
    if device is None:
        device = local_device(rank)
    costs = [flop_alg(n) * iterations for n in Ns]
    mine = partition(costs, world)[rank]
    res = runner([ps[i] for i in mine], [Ns[i] for i in mine], iterations, device) if mine else []
    records = [(i,) + tuple(r) for i, r in zip(mine, res)]
    if gather is None:
        return records
    everything = gather(records)
    if rank != 0:
        return None
    merged = sorted((rec for part in everything for rec in part), key=lambda x: x[0])
    if [r[0] for r in merged] != list(range(len(ps))):
        raise RuntimeError("sharded batch lost or duplicated tests")
    return [tuple(r[1:]) for r in merged]


def gpu_runner(ps: list[int], Ns: list[int], iterations: int, device: int):
    """Runner over one gl_batch on `device` (this rank's GPU)."""
    import gpulucas_gb300 as gl
    with gl.Batch(ps, Ns, device=device) as b:
        b.iterate(iterations, check=False)
        out = []
        for i in range(len(ps)):
            r, st = b.result(i)
            out.append((r.res64, st, r.max_roundoff))
        return out
