"""The reference's own recorded full tests, reproduced on the GPU.

gpuLucas.cu:98-108 records complete Lucas-Lehmer tests of three Mersenne primes at these
FFT lengths (the only known answers the reference itself holds):

* M859433 at N = 49152 (2^14 3, word sizes 17/18),
* M1257787 at N = 65536 (2^16, 19/20),
* M3021377 at N = 163840 (2^15 5, 18/19).

The three run together: one batch over all three plans until the shortest finishes, then
a batch over the other two, then the last alone (each test's iteration count is its own
p - 2).  Each must end after exactly p - 2 iterations with residue 0 (the exact zero
test), Res64 0, and a maximum round-off below the 0.4 limit.
"""
import pytest

pytestmark = pytest.mark.gpu

RECORDED = [(859433, 49152), (1257787, 65536), (3021377, 163840)]


def test_reference_recorded_primes(gl):
    plans = [gl.Plan(p, N) for p, N in RECORDED]
    try:
        live = list(range(len(RECORDED)))
        done = 0
        maxerr = [0.0] * len(RECORDED)
        results = {}
        while live:
            target = min(RECORDED[i][0] - 2 for i in live)
            with gl.Batch(plans=[plans[i] for i in live]) as b:
                rep = b.iterate(target - done)
                assert rep.status == 0 and rep.iterations == target - done
                for slot, i in enumerate(live):
                    r, st = b.result(slot)
                    assert st == 0 and r.iterations == target
                    maxerr[i] = max(maxerr[i], r.max_roundoff)
                    if RECORDED[i][0] - 2 == target:
                        results[i] = r
            done = target
            live = [i for i in live if i not in results]
        for i, (p, N) in enumerate(RECORDED):
            r = results[i]
            assert (r.p, r.N, r.iterations) == (p, N, p - 2)
            assert r.is_zero and r.is_prime and r.res64 == 0, p
            assert 0.0 < maxerr[i] < 0.4, (p, maxerr[i])
    finally:
        for pl in plans:
            pl.close()
