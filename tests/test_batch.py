"""Batched tests: many exponents of different sizes advance together (one set of
launches per iteration, per-test descriptor table).  Each test must produce exactly the
products of its own single-test plan, and Res64 equal to the exact oracle."""
import numpy as np
import pytest


def test_smallest_signal_size(gl):
    # config 4's rule: smallest N = 2^a 3^b 5^c 7^d (even) with p/N <= 19.5
    for p in [100003, 1000003, 2999999]:
        N = gl.smallest_signal_size(p, 19.5)
        assert N % 2 == 0 and p / N <= 19.5
        M = N // 2
        for q in (2, 3, 5, 7):
            while M % q == 0:
                M //= q
        assert M == 1
        # nothing smaller qualifies
        for n2 in range(2, N, 2):
            m = n2 // 2
            for q in (2, 3, 5, 7):
                while m % q == 0:
                    m //= q
            if m == 1 and n2 >= 64:
                assert p / n2 > 19.5


@pytest.mark.gpu
def test_batch_matches_single_plans(gl, orc):
    ps = [100003, 12379, 1000003, 44497, 2976221, 300007, 150001]
    Ns = [5184, 640, 54432, 2048, 163840, 0, 0]
    k = 130
    with gl.Batch(ps, Ns) as b:
        rep = b.iterate(k)
        assert rep.iterations == k and rep.max_roundoff < 0.4
        for i, p in enumerate(ps):
            info = b.test_info(i)
            r, st = b.result(i)
            assert st == 0 and r.iterations == k
            assert r.res64 == orc.Exact(p).iterate(k).res64(), (p, info.N)
            with gl.Plan(p, info.N) as pl:
                pl.iterate(k)
                assert pl.res64() == r.res64


@pytest.mark.gpu
def test_batch_full_prime_run_and_members(gl, orc):
    """M4423 (prime) completes its full p - 2 iterations inside a batch; the other members,
    advanced the same 4421 iterations, match the exact oracle."""
    ps = [4423, 9689, 9941, 11213, 21701]
    k = 4423 - 2
    with gl.Batch(ps, [256, 512, 512, 640, 1024]) as b:
        b.iterate(k)
        r, st = b.result(0)
        assert st == 0 and r.is_prime and r.res64 == 0
        for i, p in enumerate(ps[1:], 1):
            r, st = b.result(i)
            assert st == 0 and r.res64 == orc.Exact(p).iterate(k).res64()
