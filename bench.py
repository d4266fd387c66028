#!/usr/bin/env python
"""bench.py -- Lucas-Lehmer iterations/s on GB300 (FP64 IBDWT, fused sm_103a kernels).

Default workload: one LL iteration of the large single test p = 43112609 at
N = 2359296 = 2^18 * 3^2 (18.27 bits/word), the length the reference quotes its own
iteration rate at (gpuLucas.cu:92-97).  A step is one iteration; the L2 cache is
flushed (512 MiB write) before every timed step (the test's state and tables, about
170 MB, exceed the 129 MB L2, but part of them would otherwise stay resident).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
reference's path (the oracle's IBDWT, all host threads) on the same workload.
Under torchrun each rank runs an independent replica of the test (a single LL test
does not shard: its FFT is global), value = iterations of all ranks / max time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LL iter/s by FFT length vs plain same-GPU form"
P3, N3 = 43112609, 2359296
BY_LENGTH = [("c1", 44497, 2048), ("c2", 2976221, 163840), ("c3", P3, N3)]
REF_PUBLISHED_ITER_S = 204.72  # gpuLucas.cu:92-96, p=42643801 at N=2359296 (GTX 480 / C2050)
L2_FLUSH_BYTES = 512 << 20
WORKLOAD = f"single LL test, one iteration per step of p={P3} at N={N3} (2^18*3^2)"


def flop_alg(N: int) -> float:
    """5 N log2 N + 4 N: real forward + inverse FFT, square, weight, unweight."""
    return 5.0 * N * math.log2(N) + 4.0 * N


def kernel_flops(N: int, W: int, H: int) -> dict:
    """flop_alg split over the three fused kernels (sums to flop_alg(N))."""
    M = N // 2
    return {
        "k_col_fwd": 5.0 * M * math.log2(H) + N,
        "k_row_sq": 10.0 * M * math.log2(W) + 10.0 * M + 2.0 * N,
        "k_col_inv": 5.0 * M * math.log2(H) + N,
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms in the background."""

    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={','.join(self.FIELDS)}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def read_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic_c3.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(kernel + " ") and "dram_bytes_per_launch=" in line:
            try:
                return float(line.split("dram_bytes_per_launch=")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


def cpu_baseline(p: int, N: int, budget_s: float = 12.0) -> dict:
    """The oracle's IBDWT (the reference's algorithm on the CPU) on all host threads,
    on a bounded sample of iterations of the same test."""
    import oracle
    threads = os.cpu_count() or 1
    o = oracle.IBDWT(p, N, threads)
    t0 = time.perf_counter()
    o.iterate(1)
    one = time.perf_counter() - t0
    k = max(2, min(2000, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    o.iterate(k)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": k / dt, "unit": "iter/s", "cores": threads, "kind": "port",
            "sample": f"{k} iterations of p={p} N={N} from S0=4 (after 1 warm-up), {dt:.1f} s"}


def run_reference(args, world: int, rank: int):
    if rank != 0:
        return
    import oracle
    threads = os.cpu_count() or 1
    o = oracle.IBDWT(P3, N3, threads)
    for _ in range(max(1, args.warmup)):
        o.iterate(1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.iterate(1)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: the LL sequence from S0=4 (no dataset)",
        "config": {"workload": WORKLOAD, "p": P3, "N": N3,
                   "implementation": "CPU IBDWT restatement of the reference path (oracle/ibdwt_oracle.c), "
                                     "all host threads"},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timed iterations after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ref_cufft_leg(dev: int) -> dict:
    """Baseline leg: the reference program itself (gpuLucas.cu with cuFFT, built for sm_103a
    by oracle/build_ref.py) on the same GPU, non-verbose, timed by its own checkpoint lines
    (cudaEvents between checkpoints, one checkpoint write per interval; the second interval
    is reported, the first includes cuFFT's first calls)."""
    try:
        from oracle import refrun
    except Exception as e:  # pragma: no cover
        return {"unavailable": f"oracle import failed: {e}"}
    if not refrun.available():
        return {"unavailable": "reference program not built (no reference sources staged)"}
    out = {"program": "gpuLucas -d DEV -f N -c K p (reference sources, patched only for safety and CUDA 13; "
                      "cuFFT D2Z/Z2D + 5 kernels per iteration)",
           "timing": "ms/iter printed at its 2nd checkpoint line: wall time of K iterations between two "
                     "checkpoints by cudaEvents, one checkpoint write included; L2 warm (continuous run)"}
    # intervals long enough that the one checkpoint write per interval (N doubles to disk)
    # costs well under 1 % of the interval
    for name, p, N, every in (("c2", 2976221, 163840, 40000), ("c3", P3, N3, 12000)):
        try:
            r = refrun.run(p, N, every=every, checkpoints=2, verbose=False, timeout=600, device=dev)
            ms = r.ms_per_iter(-1)
            out[name] = {"p": p, "N": N, "iterations_per_interval": every, "ms_per_iter": ms,
                         "iter_s": 1e3 / ms, "ms_per_iter_first_interval": r.ms_per_iter(0),
                         "wall_s": r.wall_s}
        except Exception as e:
            out[name] = {"unavailable": f"{type(e).__name__}: {str(e).splitlines()[0][:200]}"}
    out["c1"] = {"unavailable": "refused by the reference: p/N = 21 (gpuLucas.cu:327-331)"}
    return out


def rate(gl, p, N, mode, seconds=0.4, device=0):
    """Continuous (L2-warm) iterations/s of one form, for the by-length table."""
    with gl.Plan(p, N, mode=mode, device=device, check_every=1 << 30) as pl:
        pl.iterate(8)
        k = 8
        while True:
            rep = pl.iterate(k)
            if rep.ms * 1e-3 >= seconds or k >= 1 << 20:
                return k / (rep.ms * 1e-3), rep.max_roundoff
            k *= 2


def run_ours(args, world: int, rank: int, local: int):
    import numpy as np
    import torch

    import gpulucas_gb300 as gl

    dev = local
    torch.cuda.set_device(dev)
    peak = gl.probe_fp64_peak(dev, 400.0)
    bfly = gl.probe_fp64_butterfly(dev, 400.0)
    plan = gl.Plan(P3, N3, device=dev, check_every=1 << 30)
    info = plan.info
    stream = torch.cuda.ExternalStream(plan.stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            flush.fill_(i & 0xFF)
            plan.enqueue(1)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(dev)
    sampler.start()
    time.sleep(0.25)
    barrier(world)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed_steps")  # lets a profiler select the timed launches
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            starts[i].record(stream)
            plan.enqueue(1)
            ends[i].record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    status = plan.sync_status(check=False)
    total_ms_max = dist_max(total_ms, world)
    value = world * args.steps / (total_ms_max * 1e-3)

    # per-kernel device time and the roofline of the dominant kernel
    prof = plan.profile_kernels(30)
    kf = kernel_flops(N3, info.fft_w, info.fft_h)
    dom = max(prof, key=prof.get)
    achieved = kf[dom] / (prof[dom] * 1e-3) / 1e12
    iter_ms = sum(prof.values())

    # end to end through the C ABI with pinned host buffers, every step: H2D of the state,
    # one iteration, D2H of the state and the round-off status, one synchronisation.  The
    # headline uses the carry-added words (gl_iterate_host_words, 4 bytes per word); the
    # carry-save pair (gl_iterate_host, int32 digit + int8 carry) is reported beside it.
    digit = torch.empty(N3, dtype=torch.int32).pin_memory()
    hi = torch.empty(N3, dtype=torch.int8).pin_memory()
    words = torch.empty(N3, dtype=torch.int32).pin_memory()
    L = gl.lib
    h = plan._h
    rc = L.gl_get_carry_state(h, ctypes.c_void_p(digit.data_ptr()), ctypes.c_void_p(hi.data_ptr()))
    assert rc == 0, rc
    words.copy_(digit + torch.roll(hi.to(torch.int32), 1))
    e2e_steps = max(50, min(200, args.steps // 4))
    rep = gl.IterReport()

    def timed(call):
        for _ in range(2):  # untimed: builds the step's graph (pinned buffers) and warms the path
            rc = call()
            assert rc == 0, rc
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            rc = call()
            assert rc == 0, rc
        return dist_max(time.perf_counter() - t0, world)

    wptr = ctypes.c_void_p(words.data_ptr())
    dptr, hptr = ctypes.c_void_p(digit.data_ptr()), ctypes.c_void_p(hi.data_ptr())
    e2e_s = timed(lambda: L.gl_iterate_host_words(h, wptr, 1, wptr, ctypes.byref(rep)))
    cs_s = timed(lambda: L.gl_iterate_host(h, dptr, hptr, 1, dptr, hptr, ctypes.byref(rep)))
    e2e = {"value": world * e2e_steps / e2e_s, "unit": "iter/s", "h2d_bytes_per_step": N3 * 4,
           "d2h_bytes_per_step": N3 * 4 + 16, "steps": e2e_steps,
           "path": "gl_iterate_host_words(plan, words, 1): H2D of the state as carry-added words "
                   "(digit[j] + hi[j-1], int32), one iteration, D2H of the words and the round-off status "
                   "(stored by the dicing kernel into the mapped pinned buffer), one synchronisation",
           "carry_save_pair": {"value": world * e2e_steps / cs_s, "unit": "iter/s",
                               "h2d_bytes_per_step": N3 * 5, "d2h_bytes_per_step": N3 * 5 + 16,
                               "path": "gl_iterate_host(plan, digit, hi, 1): int32 digit + int8 carry, "
                                       "stored by the dicing kernel into the mapped pinned buffers"}}
    plan.close()

    line = {
        "impl": "gpulucas_gb300", "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / REF_PUBLISHED_ITER_S / world, "dtype": "f64",
        "data": "synthetic: the LL sequence from S0=4 (no dataset)",
        "config": {"workload": WORKLOAD,
                   "p": P3, "N": N3, "fft": f"{info.fft_h} x {info.fft_w}", "parallelism": "replicas",
                   "layout": {"radix_h": [r for r in info.radix_h if r], "radix_w": [r for r in info.radix_w if r],
                              "column_variant": info.col_variant, "row_variant": info.row_variant,
                              "threads_col": info.threads_col,
                              "threads_row": info.threads_row},
                   "l2": "flushed before every timed step (512 MiB write); the test's ~170 MB of state and "
                         "tables exceed the 129 MB L2 anyway",
                   "vs_baseline_note": "reference's published 204.72 iter/s at N=2359296 (GTX 480/C2050)"},
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": read_traffic(dom),
                     "peak_source": "measured live: DFMA probe (gl_probe_fp64_peak); MEASURED_PEAKS.json has "
                                    "no FP64 figure",
                     "algorithmic_flops_per_launch": kf[dom], "kernel_ms": prof,
                     "butterfly_issue": {"fp64_instr_per_s": bfly, "of_dfma_probe": bfly / (peak * 0.5e12),
                                         "note": "FP64 issue rate of the line DFTs' twiddled radix-8 butterfly "
                                                 "from registers (gl_probe_fp64_butterfly), beside the DFMA "
                                                 "probe's rate (peak/2 instructions per second)"},
                     "iteration_flop_alg": flop_alg(N3),
                     "iteration_tflops": flop_alg(N3) / (iter_ms * 1e-3) / 1e12,
                     "hbm_gbs_alg": 16.0 * N3 / (iter_ms * 1e-3) / 1e9},
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": args.steps * plan_launches(gl),
        "max_roundoff": status.max_roundoff,
    }
    if rank == 0 and world == 1:
        by = {}
        for name, p, N in BY_LENGTH:
            f, ef = rate(gl, p, N, gl.MODE_FUSED, device=dev)
            pl_, ep = rate(gl, p, N, gl.MODE_PLAIN, device=dev)
            by[name] = {"p": p, "N": N, "fused_iter_s": f, "plain_iter_s": pl_, "fused_over_plain": f / pl_,
                        "fused_max_roundoff": ef, "plain_max_roundoff": ep, "l2": "warm (continuous run)"}
        if args.ref_cufft:
            ref = ref_cufft_leg(dev)
            line["ref_cufft"] = ref
            for name in ("c2", "c3"):
                if "iter_s" in ref.get(name, {}):
                    by[name]["ref_cufft_iter_s"] = ref[name]["iter_s"]
                    by[name]["fused_over_ref_cufft"] = by[name]["fused_iter_s"] / ref[name]["iter_s"]
            if "iter_s" in ref.get("c3", {}):
                line["value_over_ref_cufft"] = value / world / ref["c3"]["iter_s"]
        line["by_fft_length"] = by
        line["cpu_baseline"] = cpu_baseline(P3, N3)
        if args.batched_iters > 0:
            line["batched"] = batched_leg(gl, dev, args.batched_iters)
        if args.serve_window > 0:
            line["served"] = served_leg(gl, dev, args.serve_window)
    if world > 1 and args.batched_iters > 0:
        sb = sharded_batched_leg(gl, dev, args.batched_iters, rank, world)
        if rank == 0:
            line["batched"] = sb
    if rank == 0:
        print(json.dumps(line), flush=True)


def sharded_batched_leg(gl, dev: int, iters: int, rank: int, world: int) -> dict:
    """The batched configuration sharded over the ranks (one GPU each): each rank advances
    the tests shard.partition gives it (by modelled FP64 work) in its own batch; the
    records are gathered once at the end (all_gather_object, no data-path collective).
    tests/h = all tests / the slowest rank's device time."""
    import torch.distributed as dist

    from gpulucas_gb300 import shard, workloads
    ps = workloads.batch_exponents()
    Ns = [gl.smallest_signal_size(p, 19.5) for p in ps]
    mine = shard.partition([shard.flop_alg(n) * iters for n in Ns], world)[rank]
    b = gl.Batch([ps[i] for i in mine], [Ns[i] for i in mine], device=dev, check_every=1000) if mine else None
    barrier(world)
    ms = b.iterate(iters, check=False).ms if b else 0.0
    recs = []
    if b:
        for j, i in enumerate(mine):
            r, st = b.result(j)
            recs.append((i, r.res64, st, r.max_roundoff))
        b.close()
    t = dist_max(ms * 1e-3, world)
    parts = [None] * world
    dist.all_gather_object(parts, recs)
    merged = sorted((x for part in parts for x in part), key=lambda x: x[0])
    if [x[0] for x in merged] != list(range(len(ps))):
        raise RuntimeError("sharded batch lost or duplicated tests")
    return {
        "workload": f"{len(ps)} primes drawn uniformly from [1e5, 3e6] (numpy default_rng(4)), smallest "
                    f"7-smooth even N with p/N <= 19.5, {iters} iterations from S0=4, sharded by test over "
                    f"{world} ranks",
        "tests": len(ps), "iterations": iters, "ranks": world, "scaling": "strong (fixed 256-test batch)",
        "tests_per_rank": [len(p) for p in shard.partition([shard.flop_alg(n) * iters for n in Ns], world)],
        "seconds": t, "tests_per_h": len(ps) / t * 3600.0,
        "tflops_alg": sum(flop_alg(N) for N in Ns) * iters / t / 1e12,
        "max_roundoff": max(x[3] for x in merged), "failed": sum(1 for x in merged if x[2] != 0),
        "gpu_launches_per_rank": 3 * iters,
    }


def batched_leg(gl, dev: int, iters: int) -> dict:
    """The batched configuration: 256 seeded prime exponents in [1e5, 3e6], each at the
    smallest N = 2^a 3^b 5^c 7^d keeping <= 19.5 bits/word, advanced together for
    `iters` iterations (one set of three launches per iteration, 64-iteration graphs).
    Compared with the same tests run one at a time, in the plain and the fused form, from
    each form's measured ms/iteration at each N."""
    from gpulucas_gb300 import serve, workloads
    ps = workloads.batch_exponents()
    Ns = [gl.smallest_signal_size(p, 19.5) for p in ps]
    t0 = time.perf_counter()
    b = gl.Batch(ps, Ns, device=dev, check_every=1000)
    build_s = time.perf_counter() - t0
    import torch
    torch.cuda.nvtx.range_push("batched_steps")  # lets a profiler select the batch's launches
    rep = b.iterate(iters, check=False)
    torch.cuda.nvtx.range_pop()
    status = [b.test_status(i) for i in range(len(ps))]
    info = b.info
    b.close()
    t = rep.ms * 1e-3
    flop = sum(flop_alg(N) for N in Ns) * iters
    pairs = list(zip(ps, Ns))
    plain = serve.measure_ms_per_iter(pairs, gl.MODE_PLAIN, device=dev, iters=200)
    fused = serve.measure_ms_per_iter(pairs, gl.MODE_FUSED, device=dev, iters=200)
    seq_plain = sum(plain[N] for N in Ns) * iters * 1e-3
    seq_fused = sum(fused[N] for N in Ns) * iters * 1e-3
    # measured check of the model: 16 members spread over the length range, run one at a
    # time for the batch's iterations in each form
    order = sorted(range(len(ps)), key=lambda i: Ns[i])
    sub = [order[i * (len(order) - 1) // 15] for i in range(16)]
    check = {}
    for name, mode, ms in (("plain", gl.MODE_PLAIN, plain), ("fused", gl.MODE_FUSED, fused)):
        meas = sum(serve.run_sequential([(ps[i], Ns[i], iters) for i in sub], mode, device=dev))
        model = sum(ms[Ns[i]] for i in sub) * iters * 1e-3
        check[name] = {"tests": len(sub), "model_s": model, "measured_s": meas, "measured_over_model": meas / model}
    return {
        "workload": f"{len(ps)} primes drawn uniformly from [1e5, 3e6] (numpy default_rng(4)), smallest "
                    f"7-smooth even N with p/N <= 19.5, {iters} iterations from S0=4",
        "tests": len(ps), "iterations": iters, "N_range": [min(Ns), max(Ns)],
        "seconds": t, "tests_per_h": len(ps) / t * 3600.0, "iter_s_per_test": iters / t,
        "tflops_alg": flop / t / 1e12,
        "max_roundoff": max(e for e, _ in status), "failed": sum(1 for _, st in status if st != 0),
        "plan_build_s": build_s, "col_units": info.col_units, "row_units": info.row_units,
        "gpu_launches": 3 * iters,
        "sequential_plain_s": seq_plain, "sequential_plain_tests_per_h": len(ps) / seq_plain * 3600.0,
        "sequential_fused_s": seq_fused, "sequential_fused_tests_per_h": len(ps) / seq_fused * 3600.0,
        "speedup_vs_sequential_plain": seq_plain / t, "speedup_vs_sequential_fused": seq_fused / t,
        "sequential_note": "one test at a time: sum over tests of iterations x the form's ms/iteration at "
                           "that N, measured over 200 L2-warm iterations per distinct N (CUDA events)",
        "sequential_check": check,
    }


def served_leg(gl, dev: int, window: int) -> dict:
    """The served configuration: the first `window` requests of the seeded Poisson stream
    (mean 50/s; 80% Res64 checks after 5000 iterations with p log-uniform in [1e5, 5e7],
    20% full tests with p log-uniform in [1e5, 2e6]), served in real time with continuous
    batching against a 150 GB HBM budget, each test at gl_fast_signal_size's length.  The stream is far over one GPU's capacity, so
    the window is finite and the server runs saturated until it drains.  Compared with
    the same requests run one at a time in arrival order (plain and fused form, from each
    form's measured ms/iteration at each N)."""
    from gpulucas_gb300 import serve, workloads
    reqs = workloads.serving_requests(window)
    srv = serve.Server(device=dev, hbm_budget_bytes=150e9)
    done = srv.run(reqs, realtime=True)
    ours = serve.latency_summary(done)
    Nmap = {c.rid: c.N for c in done}
    pairs = [(r.p, Nmap[r.rid]) for r in reqs]
    out = {
        "workload": f"first {window} requests of the seeded stream (numpy default_rng(5)): Poisson arrivals "
                    "mean 50/s, 80% Res64 after k=5000 with p log-uniform prime in [1e5, 5e7], 20% full "
                    "p-2 tests with p log-uniform prime in [1e5, 2e6]; 150 GB HBM budget; real time",
        "requests": window, "full_tests": sum(r.full for r in reqs),
        "errors": sum(1 for c in done if c.status != 0),
        "restarts_at_larger_length": sum(c.attempts - 1 for c in done),
        "length_rule": "gl_fast_signal_size(p, 0.2): within 20 % above the length with "
                       "p/N <= 19.2 - 0.26 log2(N/163840), odd part 1 or 3 preferred",
        "primes_found": [c.p for c in done if c.is_prime],
        "max_roundoff": max(c.max_roundoff for c in done),
        "tflops_alg": srv.stats["flop"] / srv.stats["wall_s"] / 1e12,
        "peak_live": srv.stats["peak_live"], "peak_hbm_bytes": srv.stats["peak_bytes"],
        "steps": srv.stats["steps"], "batch_rebuilds": srv.stats["rebuilds"], "lanes": srv.stats["lanes"],
    }
    out.update({k: v for k, v in ours.items()})
    checks = [r for r in reqs if not r.full][:12]
    for name, mode in (("plain", gl.MODE_PLAIN), ("fused", gl.MODE_FUSED)):
        ms = serve.measure_ms_per_iter(pairs, mode, device=dev, iters=200)
        seq = serve.latency_summary(serve.sequential_schedule(reqs, lambda r: ms[Nmap[r.rid]]))
        out[f"sequential_{name}"] = {k: seq[k] for k in ("tests_per_h", "p50_s", "p99_s", "makespan_s")}
        # measured check of the model on the first 12 Res64 checks, run one at a time
        meas = sum(serve.run_sequential([(r.p, Nmap[r.rid], r.iterations) for r in checks], mode, device=dev))
        model = sum(r.iterations * ms[Nmap[r.rid]] for r in checks) * 1e-3
        out[f"sequential_{name}"]["check"] = {"requests": len(checks), "model_s": model, "measured_s": meas,
                                              "measured_over_model": meas / model}
        if mode == gl.MODE_FUSED:
            out["lead_lane_slowdown"] = serve.lane_slowdown(done, ms, "lead")
            out["lead_lane_slowdown"]["note"] = ("in-mix time (admission to completion) over alone time "
                                                 "(iterations x fused ms/iteration at that N)")
    out["speedup_tests_per_h_vs_sequential_plain"] = ours["tests_per_h"] / out["sequential_plain"]["tests_per_h"]
    out["sequential_note"] = ("one test at a time in arrival order: iterations x the form's ms/iteration at "
                              "that N, measured over 200 L2-warm iterations per distinct N (CUDA events)")
    return out


def plan_launches(gl) -> int:
    return 3  # fused form: k_col_fwd, k_row_sq, k_col_inv per iteration


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--batched-iters", type=int, default=10000,
                    help="iterations of the 256-test batched leg (0: skip)")
    ap.add_argument("--serve-window", type=int, default=64, help="requests in the served leg (0: skip)")
    ap.add_argument("--ref-cufft", type=int, default=1,
                    help="1: time the reference cuFFT program on the same GPU (baseline leg); 0: skip")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        args.steps = min(args.steps, 200)
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
