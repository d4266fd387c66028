"""The configurations at their full sizes on the GPU (minutes, not seconds).

* Config 2: p = 2976221 at N = 163840 = 2^15 5, the full p - 2 iterations: residue 0
  (2^2976221 - 1 is prime), max round-off reported and below the 0.4 limit.
* Config 4: the 256 seeded exponents in [1e5, 3e6], each at the smallest 7-smooth even N
  with p/N <= 19.5, advanced together for 10000 iterations: every test within the
  round-off limit, and the Res64 of six of them equal to the golden values both oracles
  agree on (tests/golden/res64_batch.json).
"""
import json
import os

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_config2_full_run_is_prime(gl):
    with gl.Plan(2976221, 163840) as pl:
        r = pl.mersenne_test(0)
    assert r.iterations == 2976219
    assert r.is_prime and r.is_zero and r.res64 == 0
    assert 0.0 < r.max_roundoff < 0.4


def test_config4_batch_full_size(gl):
    from gpulucas_gb300 import workloads
    with open(os.path.join(HERE, "golden", "res64_batch.json")) as f:
        golden = {e["p"]: e for e in json.load(f)}
    ps = workloads.batch_exponents()
    Ns = [gl.smallest_signal_size(p, 19.5) for p in ps]
    with gl.Batch(ps, Ns) as b:
        rep = b.iterate(10000)
        assert rep.iterations == 10000 and rep.status == 0 and rep.max_roundoff < 0.4
        seen = 0
        for i, p in enumerate(ps):
            r, st = b.result(i)
            assert st == 0 and r.iterations == 10000 and r.max_roundoff < 0.4
            if p in golden:
                e = golden[p]
                assert (r.N, f"{r.res64:016x}") == (e["N"], e["res64"]), p
                seen += 1
    assert seen == len(golden) >= 6
