"""Serving: continuous batching of Lucas-Lehmer requests on one GPU.

The request loop is the library's C++ server (gl_server_* in include/gpulucas.h): a
background thread admits submitted requests against an HBM budget and a slot limit,
builds each test's plan on worker threads, and advances the live tests in two batches on
two streams -- the chain lane (the device's highest stream priority) for full tests and
long requests, whose latency is a chain of dependent iterations too small to fill the
GPU, and the bulk lane for the rest, which soaks up the SMs the chain lane leaves idle;
the chain test with the most iterations left runs alone in a lead lane at the highest
priority, since the longest dependent chain sets the makespan.
A lane's batch is rebuilt from the live plans when its membership changes; every step is
bounded by `step_ms` of GPU time and by the next completion or Res64 checkpoint, so an
arrival waits at most one step.  A test whose round-off reaches the limit restarts from
S0 = 4 at the next larger FFT length (the reference aborts such a run,
gpuLucas.cu:1470-1479).  Residues stay on the device; a finished test reports its Res64
and zero test and frees its memory.

FFT lengths come from gl_fast_signal_size (within 20 % above the round-off-safe length,
the fastest kind of length), or from a fixed bits/word bound when `max_bits_per_word` is
given.  This module drives that server from Python: `Server.run` submits a request list in real
time (each request at its arrival time) or all at once, and collects the completions.
An engine object (see `PyEngine`) can stand in for the GPU so the scheduling logic runs
on the CPU in the tests.  The reference runs one test per process (gpuLucas.cu:374-639)
and has no server.

Results do not depend on co-scheduling: each test keeps its own tables and state, the
batched kernels compute exactly what the test's own fused kernels compute, and the
integer products after rounding do not depend on the FFT layout while the round-off
stays below 0.5.
"""
from __future__ import annotations

import ctypes
import itertools
import math
import statistics
import time
from dataclasses import dataclass, field
from typing import Callable, Iterable, Sequence

from .workloads import Request

GL_OK = 0
GL_ERR_NOMEM = -5      # request can never fit the HBM budget
GL_ERR_ROUNDOFF = -6
GL_ERR_STATE = -11


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


class PyEngine:
    """A gl_server_engine whose calls go to a Python object with the methods
    signal_size(p, max_bits_per_word | None, above) -> N, footprint(p, N) -> bytes,
    create(p, N) -> test, destroy(test), batch(tests, high_priority) -> batch,
    close_batch(batch), start(batch, iters), ready(batch) -> bool,
    finish(batch) -> [(max_roundoff, status)] in test order, res64(test) -> (res64, is_zero).
    Objects are passed to the server as integer handles."""

    def __init__(self, impl):
        import gpulucas_gb300 as gl
        self.gl = gl
        self.impl = impl
        self.objs: dict[int, object] = {}
        self.ids = itertools.count(1)   # callbacks come from several server threads
        self.error: BaseException | None = None

        def guard(fn, fail=GL_ERR_STATE):
            def wrapped(*a):
                try:
                    return fn(*a)
                except BaseException as e:  # noqa: BLE001 - reported after the run
                    if self.error is None:
                        self.error = e
                    return fail
            return wrapped

        def put(obj) -> int:
            h = next(self.ids)
            self.objs[h] = obj
            return h

        def signal_size(ctx, p, bits, above, N):
            N[0] = int(impl.signal_size(p, bits if bits > 0 else None, above))
            return GL_OK

        def footprint(ctx, p, N, out):
            out[0] = int(impl.footprint(p, N))
            return GL_OK

        def create(ctx, p, N, out):
            out[0] = put(impl.create(p, N))
            return GL_OK

        def destroy(ctx, h):
            impl.destroy(self.objs.pop(h))

        def batch(ctx, tests, n, high, out):
            out[0] = put(impl.batch([self.objs[tests[i]] for i in range(n)], bool(high)))
            return GL_OK

        def close_batch(ctx, h):
            impl.close_batch(self.objs.pop(h))

        def start(ctx, h, k):
            impl.start(self.objs[h], int(k))
            return GL_OK

        def ready(ctx, h):
            return 1 if impl.ready(self.objs[h]) else 0

        def finish(ctx, h, n, err, st):
            res = impl.finish(self.objs[h])
            for i in range(n):
                err[i], st[i] = float(res[i][0]), int(res[i][1])
            return GL_OK

        def res64(ctx, h, r, z):
            a, b = impl.res64(self.objs[h])
            r[0], z[0] = int(a), int(bool(b))
            return GL_OK

        e = gl.ServerEngine()
        e.ctx = None
        # the CFUNCTYPE objects must outlive the server: keep them on self
        self._cbs = [gl.ENGINE_SIGNAL_SIZE(guard(signal_size)), gl.ENGINE_FOOTPRINT(guard(footprint)),
                     gl.ENGINE_CREATE(guard(create)), gl.ENGINE_DESTROY(guard(destroy, None)),
                     gl.ENGINE_BATCH(guard(batch)), gl.ENGINE_CLOSE_BATCH(guard(close_batch, None)),
                     gl.ENGINE_START(guard(start)), gl.ENGINE_READY(guard(ready)), gl.ENGINE_FINISH(guard(finish)),
                     gl.ENGINE_RES64(guard(res64))]
        (e.signal_size, e.footprint, e.create, e.destroy, e.batch, e.close_batch, e.start, e.ready, e.finish,
         e.res64) = self._cbs
        self.struct = e


class Server:
    """Options of gl_server_opts; `engine` None runs on the GPU `device`."""

    def __init__(self, engine=None, hbm_budget_bytes: float = 150e9, max_active: int = 512, step_ms: float = 50.0,
                 checkpoint_every: int = 100_000, max_bits_per_word: float | None = None, retries: int = 2,
                 chain_iterations: int = 100_000, lanes: int = 3, build_threads: int = 2, device: int = 0,
                 error_limit: float = 0.4, check_every: int = 1000):
        import gpulucas_gb300 as gl
        self.gl = gl
        o = gl.ServerOpts()
        gl.lib.gl_server_default_opts(ctypes.byref(o))
        o.device, o.hbm_budget_bytes, o.max_active, o.step_ms = device, float(hbm_budget_bytes), max_active, step_ms
        o.checkpoint_every, o.retries, o.chain_iterations = checkpoint_every, retries, chain_iterations
        o.max_bits_per_word = 0.0 if max_bits_per_word is None else float(max_bits_per_word)
        o.lanes, o.build_threads, o.error_limit, o.check_every = lanes, build_threads, error_limit, check_every
        self.opts = o
        self.engine = PyEngine(engine) if engine is not None else None
        self.stats: dict = {}

    def run(self, requests: Iterable[Request], realtime: bool = True, poll_ms: float = 2.0) -> list[Completion]:
        """Serve `requests`: with realtime, each is submitted when the wall clock since
        the start reaches its arrival time; otherwise all are submitted at once.
        Returns one Completion per request in completion order (times in seconds since
        the server started; arrival_s is the submission time)."""
        gl = self.gl
        reqs = sorted(requests, key=lambda r: (r.arrival_s, r.rid))
        by_id = {r.rid: r for r in reqs}
        h = ctypes.c_void_p()
        eng = ctypes.byref(self.engine.struct) if self.engine is not None else None
        gl._check(gl.lib.gl_server_create(ctypes.byref(self.opts), eng, ctypes.byref(h)), "server create")
        out: list[Completion] = []
        buf = (gl.Completion * 64)()
        n = ctypes.c_int()
        err = GL_OK
        try:
            t0 = time.perf_counter()
            i = 0
            while len(out) < len(reqs):
                now = time.perf_counter() - t0
                while i < len(reqs) and (not realtime or reqs[i].arrival_s <= now):
                    r = reqs[i]
                    gl._check(gl.lib.gl_server_submit(h, r.rid, r.p, 0 if r.full else r.iterations), "submit")
                    i += 1
                wait = poll_ms
                if i < len(reqs) and realtime:
                    wait = max(0.0, min(poll_ms, (reqs[i].arrival_s - (time.perf_counter() - t0)) * 1e3))
                err = gl.lib.gl_server_poll(h, buf, 64, ctypes.byref(n), float(wait))
                if err != GL_OK:
                    break
                for c in buf[: n.value]:
                    out.append(self._completion(h, c, by_id))
            st = gl.ServerStats()
            gl.lib.gl_server_get_stats(h, ctypes.byref(st))
            names = self._lane_names()
            self.stats = dict(wall_s=st.wall_s, busy_s=max(st.lane_busy_s[i] for i in range(len(names))),
                              lanes={nm: dict(busy_s=st.lane_busy_s[i], steps=st.steps[i], rebuilds=st.rebuilds[i],
                                              peak_live=st.peak_live[i]) for i, nm in enumerate(names)},
                              steps=sum(st.steps[i] for i in range(len(names))),
                              rebuilds=sum(st.rebuilds[i] for i in range(len(names))),
                              peak_live=max(st.peak_live[i] for i in range(len(names))), peak_bytes=st.peak_bytes,
                              flop=st.flop_alg)
        finally:
            rc = gl.lib.gl_server_destroy(h)
        if self.engine is not None and self.engine.error is not None:
            raise self.engine.error
        gl._check(err if err != GL_OK else rc, "server")
        return out

    def _lane_names(self):
        n = self.opts.lanes
        return ["lead", "chain", "bulk"] if n >= 3 else (["chain", "bulk"] if n == 2 else ["all"])

    def _completion(self, h, c, by_id) -> Completion:
        gl = self.gl
        cps = []
        if c.n_checkpoints:
            its = (ctypes.c_int64 * c.n_checkpoints)()
            res = (ctypes.c_uint64 * c.n_checkpoints)()
            k = ctypes.c_int()
            gl._check(gl.lib.gl_server_checkpoints(h, c.id, its, res, c.n_checkpoints, ctypes.byref(k)),
                      "checkpoints")
            cps = [(int(its[j]), int(res[j])) for j in range(k.value)]
        lane = self._lane_names()[c.lane]
        return Completion(int(c.id), int(c.p), int(c.N), int(c.iterations), bool(c.full), float(c.arrival_s),
                          float(c.admit_s), float(c.done_s), int(c.res64), bool(c.is_zero), bool(c.is_prime),
                          float(c.max_roundoff), int(c.status), cps, int(c.attempts), lane)


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


def run_sequential(tests: Sequence[tuple[int, int, int]], mode: int, device: int = 0) -> list[float]:
    """Run (p, N, iterations) tests one at a time, each from S0 = 4 in its own plan, and
    return each one's device time in seconds (the library's CUDA-event timing of its
    iterations).  The measured check of the one-test-at-a-time comparators."""
    import gpulucas_gb300 as gl
    out = []
    for p, N, iters in tests:
        with gl.Plan(p, N, mode=mode, device=device) as pl:
            pl.reset()
            rep = pl.iterate(iters, check=False)
            out.append(rep.ms * 1e-3)
    return out


def lane_slowdown(done: Sequence[Completion], ms_per_iter: dict[int, float], lane: str = "lead") -> dict:
    """In-mix time (admission to completion) over alone time (iterations x the fused
    form's ms/iteration at that N) of the tests that ran in `lane`."""
    r = [(c.done_s - c.admit_s) / (c.iterations * ms_per_iter[c.N] * 1e-3)
         for c in done if c.lane == lane and c.status == GL_OK and c.N in ms_per_iter]
    if not r:
        return dict(tests=0)
    return dict(tests=len(r), mean=statistics.fmean(r), max=max(r), min=min(r))
