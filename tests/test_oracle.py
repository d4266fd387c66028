"""The oracle pinned before it is trusted, and the product's host tables pinned with it.

* exact NTT oracle == Python integers (S_{k+1} = S_k^2 - 2 mod 2^p - 1, S_0 = 4)
* IBDWT oracle (the reference algorithm restated) == exact oracle on Res64
* Mersenne-prime exponents give residue 0 after p - 2 iterations (the reference's only
  known answers, gpuLucas.cu:92-118)
* weights (gpuLucas.cu:673-686) and twiddles == the committed mpmath golden values,
  for the oracle's double-double code and for the product's own (gl_tables.cpp)
* bits per word: exact integer formula == the reference's double formula
  (gpuLucas.cu:688-694) on the configured sizes
* setSliceAndDice table (gpuLucas.cu:323-343), extended to ratio 21
* print_residue (gpuLucas.cu:1288-1352) restatement == exact value on random digits
"""
import ctypes
import json
import os

import numpy as np
import pytest

from gpulucas_gb300 import _build

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def hc():
    L = ctypes.CDLL(_build.HOSTCHECK)
    f64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    L.hc_weights.argtypes = [ctypes.c_int, ctypes.c_int, f64, f64]
    L.hc_twiddles.argtypes = [ctypes.c_int, f64, f64]
    L.hc_word_tables.argtypes = [ctypes.c_int, ctypes.c_int, np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"),
                                 np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")]
    return L


@pytest.mark.parametrize("p,k", [(3, 1), (5, 3), (7, 5), (89, 87), (521, 519), (4423, 300), (11213, 50)])
def test_exact_oracle_vs_python_int(orc, p, k):
    ex = orc.Exact(p).iterate(k)
    assert ex.value() == orc.lucas_lehmer_int(p, k)


@pytest.mark.parametrize("p,N,k", [(4423, 256, 300), (44497, 2048, 200), (12379, 640, 400),
                                   (100003, 5184, 100), (86243, 4096, 100), (1000003, 54432, 20)])
def test_ibdwt_oracle_vs_exact(orc, p, N, k):
    o = orc.IBDWT(p, N).iterate(k)
    digits, r, _, z = o.residue()
    assert r == orc.Exact(p).iterate(k).res64()
    assert orc.digits_to_int(p, N, digits) == orc.lucas_lehmer_int(p, k)
    assert o.maxerr < 0.4 and not o.overflow


@pytest.mark.parametrize("p,N", [(521, 32), (4423, 256), (9689, 512), (21701, 1024)])
def test_known_mersenne_primes_full_run(orc, p, N):
    o = orc.IBDWT(p, N).iterate(p - 2)
    _, r, ref_zero, exact_zero = o.residue()
    assert exact_zero and ref_zero and r == 0


def test_composite_not_zero(orc):
    o = orc.IBDWT(4441, 256).iterate(4439)   # 4441 is prime, M4441 composite
    _, r, _, z = o.residue()
    assert not z and r != 0


def test_weights_golden(orc, hc):
    for e in load("weights.json"):
        p, N = e["p"], e["N"]
        A, Ai = orc.weights(p, N)
        B = np.empty(N)
        Bi = np.empty(N)
        hc.hc_weights(p, N, B, Bi)
        for j, a, ai in zip(e["j"], e["A"], e["Ainv"]):
            assert A[j] == float.fromhex(a) and Ai[j] == float.fromhex(ai), (p, N, j)
            assert B[j] == float.fromhex(a) and Bi[j] == float.fromhex(ai), (p, N, j)


def test_twiddles_golden(orc, hc):
    for e in load("twiddles.json"):
        L = e["L"]
        w = orc.twiddles(L)
        re = np.empty(L)
        im = np.empty(L)
        hc.hc_twiddles(L, re, im)
        for t, a, b in zip(e["t"], e["re"], e["im"]):
            assert w[t].real == float.fromhex(a) and w[t].imag == float.fromhex(b), (L, t)
            assert re[t] == float.fromhex(a) and im[t] == float.fromhex(b), (L, t)


@pytest.mark.parametrize("p,N", [(44497, 2048), (2976221, 163840), (43112609, 2359296), (100003, 5184)])
def test_bits_tables(orc, hc, p, N):
    b, f = orc.bits(p, N)
    assert int(b.sum()) == p
    assert set(np.unique(b)) <= {p // N, p // N + 1}
    assert (b == orc.bits_refdouble(p, N)).all()
    b2 = np.empty(N, np.int32)
    f2 = np.empty(N, np.uint8)
    hc.hc_word_tables(p, N, b2, f2)
    assert (b == b2).all() and (f == f2).all()
    LO = p // N
    hi = (b != LO).astype(np.uint8)
    for i in range(8):
        assert (((f >> i) & 1) == np.roll(hi, i)).all()


def test_slice_depth_table(orc, gl):
    N = 1000
    expect = {21: 2, 20: 2, 19: 2, 18: 2, 17: 3, 16: 3, 15: 4, 14: 4, 13: 5, 12: 5, 11: 6, 8: 6}
    for ratio, n in expect.items():
        assert orc.slice_depth(ratio * N + 1, N) == n
        assert gl.setSliceAndDice(ratio * N + 1, N) == n
    assert orc.slice_depth(22 * N, N) == -1
    with pytest.raises(gl.GLError):
        gl.setSliceAndDice(22 * N, N)


def test_res64_normalize_vs_exact(orc):
    rng = np.random.default_rng(5)
    for p, N in [(4423, 256), (44497, 2048), (86243, 4096)]:
        b, _ = orc.bits(p, N)
        for _ in range(5):
            d = np.array([rng.integers(-(1 << (x - 1)), 1 << (x - 1)) for x in b], np.int32)
            v = orc.digits_to_int(p, N, d)
            assert orc.res64_normalize(p, N, d) == v & ((1 << 64) - 1)


def test_rebalance_preserves_value(orc):
    rng = np.random.default_rng(9)
    p, N = 44497, 2048
    b, _ = orc.bits(p, N)
    d = np.array([rng.integers(-(1 << (x - 1)), 1 << (x - 1)) for x in b], np.int32)
    h = rng.integers(-3, 4, N).astype(np.int8)
    out = orc.rebalance(p, N, d, h)
    assert orc.digits_to_int(p, N, out) == orc.carry_state_to_int(p, N, d, h)


def test_golden_res64_fixture_consistent():
    entries = load("res64.json")
    assert any(e["p"] == 44497 and e["k"] == 44495 and e["is_zero"] for e in entries)
    for e in entries:
        if e["k"] == e["p"] - 2 and e["p"] in (44497, 86243, 2976221, 43112609):
            assert e["is_zero"] and int(e["res64"], 16) == 0


def test_batch_golden_small_entries_recomputed():
    """The batched configuration's golden Res64 (k = 10000), recomputed for the two small
    exponents by the exact oracle."""
    import json
    import os

    import oracle
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "res64_batch.json")) as f:
        entries = json.load(f)
    assert len(entries) == 6 and all(e["k"] == 10000 for e in entries)
    for e in entries:
        if e["p"] < 200000:
            assert f"{oracle.Exact(e['p']).iterate(10000).res64():016x}" == e["res64"]
