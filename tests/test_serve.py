"""Serving loop: continuous batching against an HBM budget.

CPU tests drive the scheduler with an exact integer engine (Python integers) in place of
the GPU: admission under the budget and the slot limit, exact stopping at each request's
iteration count, Res64 checkpoints of full tests, round-off retirement, rejection of a
request that can never fit.  GPU tests serve a mixed window through the library and
require every result to equal the same test run alone and the exact oracle.
"""
import pytest

from gpulucas_gb300 import serve
from gpulucas_gb300.workloads import Request


class IntLL:
    """S_k mod 2^p - 1 with Python integers (the exact restatement, S_0 = 4)."""

    def __init__(self, p):
        self.p, self.M, self.s, self.iters_done = p, (1 << p) - 1, 4, 0

    def iterate(self, k):
        s, M, p = self.s, self.M, self.p
        for _ in range(k):
            s = s * s - 2 + M          # >= 0
            s = (s & M) + (s >> p)     # 2^p == 1
            s = (s & M) + (s >> p)
            if s >= M:
                s -= M
        self.s = s
        self.iters_done += k
        return self

    def res64(self):
        return self.s & 0xFFFFFFFFFFFFFFFF

    def is_zero(self):
        return self.s == 0

    def close(self):
        pass


class ExactEngine:
    """Engine interface over exact integer LL: a 'batch' is the list of live tests."""

    def __init__(self, bad=(), bytes_per_word=63):
        self.bad = set(bad)
        self.bpw = bytes_per_word
        self.live_counts = []

    def signal_size(self, p, bits, above=0):
        import gpulucas_gb300 as gl
        if above:
            return gl.smallest_signal_size(p, p / (above + 1.0))
        return gl.safe_signal_size(p) if bits is None else gl.smallest_signal_size(p, bits)

    def footprint(self, p, N):
        return self.bpw * N

    def create(self, p, N):
        return IntLL(p)

    def destroy(self, h):
        h.close()

    def batch(self, handles, high_priority):
        self.live_counts.append(len(handles))
        self.lanes_seen = getattr(self, "lanes_seen", set()) | {high_priority}
        return [list(handles), 0]

    def close_batch(self, b):
        pass

    def start(self, b, k):
        b[1] = k

    def ready(self, b):
        return True

    def finish(self, b):
        out = []
        for h in b[0]:
            h.iterate(b[1])
            out.append((0.45, serve.GL_ERR_ROUNDOFF) if h.p in self.bad else (0.1, serve.GL_OK))
        return out

    def res64(self, h):
        return h.res64(), h.is_zero()


def _exact(p, k):
    return IntLL(p).iterate(k).res64()


def test_serve_exact_results_and_budget():
    reqs = [Request(0, 0.0, 100003, 300, False), Request(1, 0.0, 4423, 4421, True),
            Request(2, 0.0, 12379, 700, False), Request(3, 0.0, 250007, 50, False),
            Request(4, 0.0, 9941, 9939, True), Request(5, 0.0, 21701, 1200, False)]
    eng = ExactEngine()
    import gpulucas_gb300 as gl
    sizes = {r.rid: gl.smallest_signal_size(r.p, 19.5) for r in reqs}
    budget = 63 * (sizes[0] + sizes[3])          # the two largest fit together, not three
    srv = serve.Server(eng, hbm_budget_bytes=budget, max_active=3, checkpoint_every=1000, step_ms=1e9,
                       max_bits_per_word=19.5)
    done = srv.run(reqs, realtime=False)
    assert sorted(c.rid for c in done) == list(range(len(reqs)))
    assert srv.stats["peak_bytes"] <= budget and max(eng.live_counts) <= 3
    assert eng.lanes_seen == {True, False}          # full tests ran in the priority lanes
    assert {c.lane for c in done if reqs[c.rid].full} <= {"lead", "chain"}
    assert "lead" in {c.lane for c in done}
    assert {c.lane for c in done if not reqs[c.rid].full} == {"bulk"}
    for c in done:
        r = reqs[c.rid]
        assert c.status == serve.GL_OK and c.iterations == r.iterations
        assert c.res64 == _exact(r.p, r.iterations), r
        if r.full:
            assert c.is_prime and c.res64 == 0          # M4423 and M9941 are prime
            assert [i for i, _ in c.checkpoints] == list(range(1000, r.iterations, 1000))
            ex = IntLL(r.p)
            for i, res in c.checkpoints:
                assert res == ex.iterate(i - ex.iters_done).res64()
        else:
            assert not c.is_prime and not c.checkpoints


def test_serve_retires_roundoff_and_rejects_oversize():
    reqs = [Request(0, 0.0, 100003, 200, False), Request(1, 0.0, 12379, 500, False),
            Request(2, 0.0, 44497, 400, False)]
    import gpulucas_gb300 as gl
    big = gl.smallest_signal_size(100003, 19.5)
    eng = ExactEngine(bad={12379})
    srv = serve.Server(eng, hbm_budget_bytes=63 * big - 1, step_ms=1e9, max_bits_per_word=19.5, retries=2)
    done = {c.rid: c for c in srv.run(reqs, realtime=False)}
    assert done[0].status == serve.GL_ERR_NOMEM and done[0].iterations == 0
    # round-off: restarted twice at larger lengths, then retired
    assert done[1].status == serve.GL_ERR_ROUNDOFF and done[1].max_roundoff >= 0.4
    assert done[1].attempts == 3 and done[1].N > gl.smallest_signal_size(12379, 19.5)
    assert done[2].status == serve.GL_OK and done[2].res64 == _exact(44497, 400) and done[2].attempts == 1


def test_serve_retry_at_larger_length_recovers():
    """A test whose round-off fails at its first length completes at the next one."""
    class OnceBad(ExactEngine):
        def create(self, p, N):
            h = super().create(p, N)
            h.first = not hasattr(self, "seen")
            self.seen = True
            return h

        def finish(self, b):
            out = []
            for h in b[0]:
                h.iterate(b[1])
                out.append((0.5, serve.GL_ERR_ROUNDOFF) if h.first else (0.1, serve.GL_OK))
            return out
    eng = OnceBad()
    srv = serve.Server(eng, step_ms=1e9)
    (c,) = srv.run([Request(0, 0.0, 21701, 300, False)], realtime=False)
    import gpulucas_gb300 as gl
    assert c.status == serve.GL_OK and c.attempts == 2 and c.N > gl.safe_signal_size(21701)
    assert c.res64 == _exact(21701, 300) and c.iterations == 300


def test_serve_realtime_arrivals_overlap():
    """Requests arriving while others run join the live set (continuous batching)."""
    reqs = [Request(i, 0.01 * i, p, 1500, False) for i, p in enumerate([4423, 9689, 9941, 11213])]
    eng = ExactEngine()
    srv = serve.Server(eng, step_ms=5.0)
    done = srv.run(reqs, realtime=True)
    assert sorted(c.rid for c in done) == [0, 1, 2, 3]
    assert max(eng.live_counts) >= 2
    for c in done:
        assert c.arrival_s <= c.admit_s <= c.done_s
        assert c.res64 == _exact(c.p, 1500)


def test_latency_summary_and_sequential_schedule():
    reqs = [Request(0, 0.0, 1, 100, False), Request(1, 0.5, 1, 100, False), Request(2, 0.6, 1, 300, False)]
    seq = serve.sequential_schedule(reqs, lambda r: 10.0)      # 10 ms / iteration
    assert [round(c.done_s, 9) for c in seq] == [1.0, 2.0, 5.0]
    s = serve.latency_summary(seq)
    assert s["completed"] == 3 and abs(s["makespan_s"] - 5.0) < 1e-9
    assert abs(s["p50_s"] - 1.5) < 1e-9 and abs(s["p99_s"] - 4.4) < 1e-9
    assert serve.percentile([1.0], 99) == 1.0


@pytest.mark.gpu
def test_serve_gpu_each_result_same_alone_and_in_mix(gl, orc):
    """A mixed window served with continuous batching: every Res64 equals the same test
    run alone (its own autotuned plan) and the exact oracle; full tests of Mersenne
    primes end with residue 0; the live set really held several tests at once."""
    reqs = [Request(0, 0.00, 100003, 600, False), Request(1, 0.01, 4423, 4421, True),
            Request(2, 0.02, 1000003, 300, False), Request(3, 0.03, 12379, 900, False),
            Request(4, 0.04, 9689, 9687, True), Request(5, 0.05, 2976221, 200, False),
            Request(6, 0.06, 300007, 1000, False), Request(7, 0.07, 11213, 11211, True),
            Request(8, 0.08, 150001, 500, False), Request(9, 0.09, 44497, 2000, False)]
    srv = serve.Server(device=0, hbm_budget_bytes=8e9, checkpoint_every=2000, step_ms=20.0)
    done = srv.run(reqs, realtime=True)
    assert sorted(c.rid for c in done) == list(range(len(reqs)))
    assert srv.stats["peak_live"] >= 3
    for c in done:
        r = reqs[c.rid]
        assert c.status == 0 and c.iterations == r.iterations and c.max_roundoff < 0.4
        exact = orc.Exact(r.p).iterate(r.iterations).res64()
        assert c.res64 == exact, r
        with gl.Plan(r.p, c.N) as pl:
            pl.reset()
            pl.iterate(r.iterations)
            assert pl.res64() == c.res64
        if r.full:
            assert c.is_prime and c.res64 == 0
            ex = orc.Exact(r.p)
            for i, res in c.checkpoints:
                assert res == ex.iterate(i - ex.iters_done).res64()


@pytest.mark.gpu
def test_describe_predicts_batch_plan_footprint(gl):
    for p in (4423, 100003, 1000003, 2976221):
        N = gl.smallest_signal_size(p, 19.5)
        est = gl.describe(p, N, batch_layout=1).device_bytes
        with gl.Plan(p, N, batch_layout=1, autotune=0) as pl:
            assert pl.info.device_bytes <= est <= 1.05 * pl.info.device_bytes + 4096, (p, N)
            assert (pl.info.fft_h, pl.info.fft_w) == (gl.describe(p, N, batch_layout=1).fft_h,
                                                      gl.describe(p, N, batch_layout=1).fft_w)


def test_serve_lead_lane_holds_longest_chain():
    """The full test with the most iterations left runs alone in the lead lane; the other
    long tests share the chain lane, the short requests the bulk lane."""
    reqs = [Request(0, 0.0, 4423, 4421, True), Request(1, 0.0, 9941, 9939, True),
            Request(2, 0.0, 9689, 9687, True), Request(3, 0.0, 12379, 300, False)]
    eng = ExactEngine()
    srv = serve.Server(eng, step_ms=1e9, checkpoint_every=0)
    done = {c.rid: c for c in srv.run(reqs, realtime=False)}
    assert done[1].lane == "lead" and done[3].lane == "bulk"
    assert {done[0].lane, done[2].lane} <= {"chain", "lead"}
    for c in done.values():
        assert c.status == serve.GL_OK and c.res64 == _exact(c.p, c.iterations)
    assert done[0].is_prime and done[1].is_prime and done[2].is_prime


def test_lane_slowdown_from_completions():
    """In-mix over alone time of the tests one lane ran (alone = iterations x ms/iteration)."""
    from gpulucas_gb300 import serve
    C = serve.Completion
    done = [C(1, 101, 4096, 1000, True, 0.0, 1.0, 3.0, 0, False, False, 0.0, 0, lane="lead"),
            C(2, 103, 8192, 2000, True, 0.0, 0.5, 4.5, 0, False, False, 0.0, 0, lane="lead"),
            C(3, 107, 4096, 500, False, 0.0, 0.0, 9.0, 0, False, False, 0.0, 0, lane="bulk")]
    r = serve.lane_slowdown(done, {4096: 1.0, 8192: 1.0}, "lead")
    assert r["tests"] == 2 and abs(r["mean"] - 2.0) < 1e-12 and r["max"] == 2.0
    assert serve.lane_slowdown(done, {4096: 1.0}, "chain") == {"tests": 0}
