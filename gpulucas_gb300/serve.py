"""Serving loop: continuous batching of Lucas-Lehmer requests on one GPU.

A request asks for the Res64 of 2^p - 1 after k iterations from S0 = 4, or for a full
p - 2 test.  Requests arrive over time; the server

* admits queued requests in arrival order while the number of live tests is below
  `max_active` and their device footprint (as `describe` predicts it) fits the HBM
  budget; a test's tables are built on a worker thread while the GPU runs the others;
* keeps every live test's state on the device and advances the live tests together, one
  set of batched launches per iteration (a gl_batch over the live plans, rebuilt only when
  the live set changes; the plans and their state are not touched by a rebuild);
* runs two such batches side by side on two streams.  The chain lane (a stream at the
  device's highest priority) holds the tests with long iteration chains (full tests and
  any request of more than `chain_iterations`): their latency is a chain of dependent
  iterations, each too small to fill the GPU, so their blocks are scheduled first.  The
  bulk lane holds the rest and soaks up the SMs the chain lane leaves idle;
* steps each lane by at most `step_ms` of GPU time, never past the next completion or
  Res64 checkpoint of its tests, so arrivals wait at most one step to be admitted;
* checks every live test's round-off after each step: a test at or above the limit stops,
  as the reference aborts (gpuLucas.cu:1470-1479), and is queued again from S0 = 4 at the
  next larger FFT length (at most `retries` times, then retired with GL_ERR_ROUNDOFF);
* records the Res64 of full tests every `checkpoint_every` iterations, and retires
  finished tests with their Res64 / zero test, freeing their memory for the queue.

FFT lengths come from gl_safe_signal_size (a host rule calibrated on the fused kernels'
measured round-off), or from a fixed bits/word bound when `max_bits_per_word` is given.

Results do not depend on co-scheduling: each test keeps its own tables and state, the
batched kernels compute exactly what the test's own fused kernels compute, and the
integer products after rounding do not depend on the FFT layout while the round-off
stays below 0.5.

The reference runs one test per process (gpuLucas.cu:374-639) and has no server; this
module is the served configuration of this library.  The engine behind the loop is a
small interface (`GpuEngine` here) so the scheduling logic can be exercised on the CPU
with an exact integer engine in the tests.
"""
from __future__ import annotations

import math
import statistics
import time
from collections import deque
from concurrent.futures import Future, ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Callable, Iterable, Sequence

from .workloads import Request

GL_OK = 0
GL_ERR_NOMEM = -5      # request can never fit the HBM budget
GL_ERR_ROUNDOFF = -6


def flop_alg(N: int) -> float:
    """5 N log2 N + 4 N: real forward + inverse FFT, square, weight, unweight."""
    return 5.0 * N * math.log2(N) + 4.0 * N


@dataclass
class Completion:
    rid: int
    p: int
    N: int
    iterations: int
    full: bool
    arrival_s: float
    admit_s: float
    done_s: float
    res64: int
    is_zero: bool
    is_prime: bool
    max_roundoff: float
    status: int
    checkpoints: list = field(default_factory=list)   # (iteration, res64) of full tests
    attempts: int = 1                                  # 1 + restarts at a larger length
    lane: str = ""

    @property
    def latency_s(self) -> float:
        return self.done_s - self.arrival_s


@dataclass
class _Live:
    req: Request
    N: int
    nbytes: int
    admit_s: float
    handle: object = None
    future: Future | None = None
    done: int = 0
    maxerr: float = 0.0
    checkpoints: list = field(default_factory=list)
    attempts: int = 1


class GpuEngine:
    """The library's fused-form plans and batches on one device."""

    def __init__(self, device: int = 0, check_every: int = 1000, error_limit: float = 0.4, batch_layout: int = 0):
        """batch_layout=0: each test keeps the layout it would have alone (cost model for
        the whole device), so a test left running alone is not slowed down; 1: the layout
        with the least total work."""
        import gpulucas_gb300 as gl
        self.gl = gl
        self.device = device
        self.layout = dict(batch_layout=int(batch_layout), autotune=0)
        self.opts = dict(device=device, check_every=check_every, error_limit=error_limit)

    def signal_size(self, p: int, max_bits_per_word: float | None, above: int = 0) -> int:
        """Length for p (larger than `above` when given)."""
        if above:
            return self.gl.smallest_signal_size(p, p / (above + 1.0))
        if max_bits_per_word is None:
            return self.gl.safe_signal_size(p)
        return self.gl.smallest_signal_size(p, max_bits_per_word)

    def footprint(self, p: int, N: int) -> int:
        return int(self.gl.describe(p, N, device=self.device, **self.layout).device_bytes)

    def create(self, p: int, N: int):
        pl = self.gl.Plan(p, N, **self.layout, **self.opts)
        pl.reset()
        return pl

    def destroy(self, handle) -> None:
        handle.close()

    def batch(self, handles: Sequence, high_priority: bool) -> object:
        return self.gl.Batch(plans=list(handles), high_priority=int(high_priority), **self.opts)

    def close_batch(self, batch) -> None:
        batch.close()

    def start(self, batch, iters: int) -> None:
        batch.enqueue(iters)

    def ready(self, batch) -> bool:
        return batch.query()

    def finish(self, batch) -> list[tuple[float, int]]:
        """Per test (max round-off so far in this batch, status) after the enqueued work."""
        batch.sync_status(check=False)
        return [batch.test_status(i) for i in range(batch.ntests)]

    def res64(self, handle) -> tuple[int, bool]:
        return handle.res64_zero()


@dataclass
class _Lane:
    name: str
    high: bool
    live: list = field(default_factory=list)
    batch: object = None
    members: tuple = ()
    iter_ms: float | None = None     # measured ms per iteration of the current members
    inflight: int = 0                # iterations enqueued and not yet collected
    t_start: float = 0.0
    busy_s: float = 0.0
    steps: int = 0
    rebuilds: int = 0
    peak_live: int = 0


class Server:
    def __init__(self, engine, hbm_budget_bytes: float = 150e9, max_active: int = 512, step_ms: float = 50.0,
                 checkpoint_every: int = 100_000, max_bits_per_word: float | None = None, retries: int = 2,
                 chain_iterations: int = 100_000, lanes: int = 2, build_threads: int = 2,
                 clock: Callable[[], float] = time.perf_counter, poll_s: float = 2e-4):
        """lanes=1 puts every test in one batch (no chain lane)."""
        self.engine = engine
        self.budget = int(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.step_ms = float(step_ms)
        self.checkpoint_every = int(checkpoint_every)
        self.bits = None if max_bits_per_word is None else float(max_bits_per_word)
        self.retries = int(retries)
        self.chain_iterations = int(chain_iterations)
        self.nlanes = 2 if lanes >= 2 else 1
        self.build_threads = max(1, int(build_threads))
        self.clock = clock
        self.poll_s = float(poll_s)
        self.stats: dict = {}

    def _lane_of(self, req: Request) -> int:
        if self.nlanes == 1:
            return 0
        return 0 if (req.full or req.iterations > self.chain_iterations) else 1

    # ------------------------------------------------------------------------
    def run(self, requests: Iterable[Request], realtime: bool = True) -> list[Completion]:
        """Serve `requests`.  With realtime, a request is visible only once the wall
        clock since the start passes its arrival time; otherwise all are queued at once
        at time 0.  Returns one Completion per request, in completion order; times are
        seconds since the start."""
        reqs = sorted(requests, key=lambda r: (r.arrival_s, r.rid))
        if not realtime:
            reqs = [Request(r.rid, 0.0, r.p, r.iterations, r.full) for r in reqs]
        eng = self.engine
        t0 = self.clock()

        def now():
            return self.clock() - t0

        incoming = deque(reqs)
        queue: deque[_Live] = deque()
        building: list[_Live] = []
        lanes = [_Lane("chain", True), _Lane("bulk", False)] if self.nlanes == 2 else [_Lane("all", False)]
        out: list[Completion] = []
        used = 0
        peak_bytes = 0
        flop_done = 0.0
        pool = ThreadPoolExecutor(self.build_threads)

        def nlive():
            return sum(len(ln.live) for ln in lanes)

        def arrive():
            t = now()
            while incoming and incoming[0].arrival_s <= t:
                r = incoming.popleft()
                N = eng.signal_size(r.p, self.bits)
                queue.append(_Live(r, N, eng.footprint(r.p, N), 0.0))

        def admit():
            nonlocal used, peak_bytes
            while queue and nlive() + len(building) < self.max_active and used + queue[0].nbytes <= self.budget:
                e = queue.popleft()
                e.admit_s = now()
                used += e.nbytes
                peak_bytes = max(peak_bytes, used)
                e.future = pool.submit(eng.create, e.req.p, e.N)
                building.append(e)
            if queue and not nlive() and not building and queue[0].nbytes > self.budget:
                e = queue.popleft()   # can never fit: reject rather than wait forever
                out.append(Completion(e.req.rid, e.req.p, e.N, 0, e.req.full, e.req.arrival_s, now(), now(),
                                      0, False, False, 0.0, GL_ERR_NOMEM, attempts=e.attempts))

        def collect(block: bool):
            for e in list(building):
                if block or e.future.done():
                    e.handle = e.future.result()
                    e.future = None
                    building.remove(e)
                    lanes[self._lane_of(e.req)].live.append(e)
                    block = False

        def retire(ln: _Lane, e: _Live, status: int):
            nonlocal used
            res, zero = eng.res64(e.handle) if status == GL_OK else (0, False)
            full_done = e.req.full and e.done == e.req.p - 2
            eng.destroy(e.handle)
            used -= e.nbytes
            if status == GL_ERR_ROUNDOFF and e.attempts <= self.retries:
                # start again from S0 = 4 at the next larger length, ahead of the queue
                N = eng.signal_size(e.req.p, self.bits, above=e.N)
                queue.appendleft(_Live(e.req, N, eng.footprint(e.req.p, N), 0.0, attempts=e.attempts + 1))
                return
            out.append(Completion(e.req.rid, e.req.p, e.N, e.done, e.req.full, e.req.arrival_s, e.admit_s, now(),
                                  res, zero, bool(full_done and zero and status == GL_OK), e.maxerr, status,
                                  e.checkpoints, e.attempts, ln.name))

        def land(ln: _Lane):
            """Collect a finished step of lane `ln`: statuses, checkpoints, retirements."""
            nonlocal flop_done
            k = ln.inflight
            st = eng.finish(ln.batch)
            dt = self.clock() - ln.t_start
            ln.busy_s += dt
            ln.iter_ms = dt * 1e3 / k
            ln.inflight = 0
            done_now = []
            for e, (err, s) in zip(ln.live, st):
                e.done += k
                e.maxerr = max(e.maxerr, err)
                flop_done += flop_alg(e.N) * k
                if s != GL_OK:
                    done_now.append((e, s))
                elif e.done >= e.req.iterations:
                    done_now.append((e, GL_OK))
                elif e.req.full and self.checkpoint_every > 0 and e.done % self.checkpoint_every == 0:
                    e.checkpoints.append((e.done, eng.res64(e.handle)[0]))
            if done_now:
                eng.close_batch(ln.batch)
                ln.batch, ln.members = None, ()
                for e, s in done_now:
                    ln.live.remove(e)
                    retire(ln, e, s)

        def launch(ln: _Lane):
            key = tuple(id(e) for e in ln.live)
            if key != ln.members:
                if ln.batch is not None:
                    eng.close_batch(ln.batch)
                ln.batch = eng.batch([e.handle for e in ln.live], ln.high)
                ln.members = key
                ln.iter_ms = None
                ln.rebuilds += 1
            ln.peak_live = max(ln.peak_live, len(ln.live))
            # bounded by the time budget, the next completion and the next checkpoint
            k = min(e.req.iterations - e.done for e in ln.live)
            for e in ln.live:
                if e.req.full and self.checkpoint_every > 0:
                    k = min(k, self.checkpoint_every - e.done % self.checkpoint_every)
            k = min(k, max(1, int(self.step_ms / ln.iter_ms)) if ln.iter_ms else 8)
            ln.t_start = self.clock()
            eng.start(ln.batch, k)
            ln.inflight = k
            ln.steps += 1

        try:
            while True:
                arrive()
                admit()
                busy = any(ln.inflight for ln in lanes)
                collect(block=not nlive() and bool(building) and not busy)
                if not nlive() and not busy:
                    if not incoming and not queue and not building:
                        break
                    if incoming and not queue and not building:
                        time.sleep(max(0.0, min(0.05, incoming[0].arrival_s - now())))
                    continue
                progressed = False
                for ln in lanes:
                    if ln.inflight and eng.ready(ln.batch):
                        land(ln)
                        progressed = True
                    if ln.live and not ln.inflight:
                        launch(ln)
                        progressed = True
                if not progressed:
                    time.sleep(self.poll_s)
        finally:
            # normal exit leaves nothing live; after an error, free what is left
            for ln in lanes:
                if ln.batch is not None:
                    if ln.inflight:
                        eng.finish(ln.batch)
                    eng.close_batch(ln.batch)
            pool.shutdown(wait=True)
            for e in building:
                if e.future is not None and e.future.exception() is None:
                    eng.destroy(e.future.result())
            for ln in lanes:
                for e in ln.live:
                    eng.destroy(e.handle)
        wall = now()
        self.stats = dict(wall_s=wall, busy_s=max(ln.busy_s for ln in lanes),
                          lanes={ln.name: dict(busy_s=ln.busy_s, steps=ln.steps, rebuilds=ln.rebuilds,
                                               peak_live=ln.peak_live) for ln in lanes},
                          steps=sum(ln.steps for ln in lanes), rebuilds=sum(ln.rebuilds for ln in lanes),
                          peak_live=max(ln.peak_live for ln in lanes), peak_bytes=peak_bytes, flop=flop_done)
        return out


# ----------------------------------------------------------------------------
def latency_summary(done: Sequence[Completion], first_arrival: float = 0.0) -> dict:
    """Completed tests/h over the makespan (first arrival to last completion) and
    completion-latency percentiles (nearest-rank)."""
    ok = [c for c in done if c.status == GL_OK]
    if not ok:
        return dict(completed=0)
    lat = sorted(c.latency_s for c in ok)
    makespan = max(c.done_s for c in ok) - first_arrival
    return dict(completed=len(ok), makespan_s=makespan, tests_per_h=3600.0 * len(ok) / makespan,
                p50_s=percentile(lat, 50), p99_s=percentile(lat, 99), mean_s=statistics.fmean(lat),
                max_s=lat[-1])


def percentile(sorted_vals: Sequence[float], q: float) -> float:
    """Nearest-rank percentile of an ascending list."""
    if not sorted_vals:
        return float("nan")
    i = max(0, min(len(sorted_vals) - 1, math.ceil(q / 100.0 * len(sorted_vals)) - 1))
    return float(sorted_vals[i])


def sequential_schedule(requests: Sequence[Request], ms_per_iter: Callable[[Request], float]) -> list[Completion]:
    """The one-test-at-a-time form: requests run in arrival order, each starting when it
    has arrived and the previous one has finished, for iterations x ms_per_iter(request)."""
    t = 0.0
    out = []
    for r in sorted(requests, key=lambda r: (r.arrival_s, r.rid)):
        start = max(t, r.arrival_s)
        t = start + r.iterations * ms_per_iter(r) / 1e3
        out.append(Completion(r.rid, r.p, 0, r.iterations, r.full, r.arrival_s, start, t, 0, False, False, 0.0,
                              GL_OK))
    return out


def measure_ms_per_iter(ps_Ns: Iterable[tuple[int, int]], mode: int, device: int = 0, iters: int = 200,
                        warmup: int = 20) -> dict[int, float]:
    """ms per iteration of a single test at each distinct N, measured with the
    library's own timing (CUDA events around `iters` iterations after `warmup`)."""
    import gpulucas_gb300 as gl
    out: dict[int, float] = {}
    for p, N in ps_Ns:
        if N in out:
            continue
        with gl.Plan(p, N, mode=mode, device=device) as pl:
            pl.reset()
            pl.iterate(warmup, check=False)
            rep = pl.iterate(iters, check=False)
            out[N] = rep.ms / iters
    return out
