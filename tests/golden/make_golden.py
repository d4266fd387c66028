"""Generate the committed golden fixtures under tests/golden/.

Run in a container with mpmath:  python tests/golden/make_golden.py [--quick | --batch]

* weights.json  -- IBDWT weights A[j] = 2^(ceil(jp/N) - jp/N) and Ainv[j] = (1/A[j])/N
  (computeWeightVectors, gpuLucas.cu:673-686) correctly rounded from 140-bit mpmath, at
  sampled j for the configured (p, N).
* twiddles.json -- exp(-2 pi i t/L) correctly rounded (mpmath cospi/sinpi).
* res64.json    -- Res64 of S_k mod 2^p - 1 (S_0 = 4) for (p, N, k).
* res64_batch.json -- the same for six of the batched configuration's 256 seeded
  exponents (workloads.batch_exponents) at its length rule (smallest 7-smooth even N with
  p/N <= 19.5) after its 10000 iterations.  Each entry is
  computed twice, by the exact NTT oracle (exact_oracle.c) and by the IBDWT oracle
  (ibdwt_oracle.c, the reference algorithm restated), and kept only when they agree.
  Entries with k = p - 2 for Mersenne-prime exponents must be 0.

Composite exponents near 2976229 are drawn from the primes in [2976221, 2996221] by
numpy.random.default_rng(2976229).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def primes_in(lo: int, hi: int):
    import sympy
    return [int(q) for q in sympy.primerange(lo, hi)]


def composite_draws(count: int):
    ps = primes_in(2976221, 2996221)
    ps = [q for q in ps if q != 2976221]
    rng = np.random.default_rng(2976229)
    idx = rng.choice(len(ps), size=count, replace=False)
    return sorted(int(ps[i]) for i in idx)


def weights_fixture():
    import mpmath
    mpmath.mp.prec = 140
    out = []
    for p, N in [(44497, 2048), (2976221, 163840), (43112609, 2359296), (100003, 5184), (1000003, 54432)]:
        rng = np.random.default_rng(p)
        js = sorted(set(list(range(0, min(N, 64))) + [int(x) for x in rng.integers(0, N, 192)] + [N - 1]))
        A, Ai = [], []
        for j in js:
            r = (-(j * p)) % N
            a = mpmath.power(2, mpmath.mpf(r) / N)
            A.append(float(a).hex())
            Ai.append(float(1 / a / N).hex())
        out.append({"p": p, "N": N, "j": js, "A": A, "Ainv": Ai})
    return out


def twiddles_fixture():
    import mpmath
    mpmath.mp.prec = 140
    out = []
    for L in [1024, 1152, 320, 81920, 1179648, 81, 168]:
        rng = np.random.default_rng(L)
        ts = sorted(set(list(range(0, min(L, 64))) + [int(x) for x in rng.integers(0, L, 128)]))
        re, im = [], []
        for t in ts:
            x = mpmath.mpf(2 * t) / L
            re.append(float(mpmath.cospi(x)).hex())
            im.append(float(-mpmath.sinpi(x)).hex())
        out.append({"L": L, "t": ts, "re": re, "im": im})
    return out


def res64_entry(p: int, N: int, k: int, threads: int = 0):
    t0 = time.time()
    ex = oracle.Exact(p, threads).iterate(k)
    r_exact = ex.res64()
    z_exact = ex.is_zero()
    ex.close()
    t1 = time.time()
    ib = oracle.IBDWT(p, N, threads).iterate(k)
    _, r_ibdwt, _, z_ibdwt = ib.residue()
    err = ib.maxerr
    ib.close()
    t2 = time.time()
    if r_exact != r_ibdwt or z_exact != z_ibdwt:
        raise SystemExit(f"oracles disagree at p={p} N={N} k={k}: {r_exact:#x} vs {r_ibdwt:#x}")
    print(f"p={p} N={N} k={k} res64={r_exact:#018x} zero={z_exact} maxerr={err:.4f} "
          f"exact {t1 - t0:.1f}s ibdwt {t2 - t1:.1f}s", flush=True)
    return {"p": p, "N": N, "k": k, "res64": f"{r_exact:016x}", "is_zero": bool(z_exact),
            "oracle_maxerr": round(err, 6)}


def batch_fixture(threads: int = 0):
    import gpulucas_gb300 as gl
    from gpulucas_gb300 import workloads
    ps = sorted(workloads.batch_exponents())
    path = os.path.join(HERE, "res64_batch.json")
    entries = []
    if os.path.exists(path):
        with open(path) as f:
            entries = json.load(f)
    have = {e["p"] for e in entries}
    for i in (0, 1, 50, 128, 200, 255):
        p = ps[i]
        if p in have:
            continue
        entries.append(res64_entry(p, gl.smallest_signal_size(p, 19.5), 10000, threads))
        with open(path, "w") as f:
            json.dump(entries, f, indent=1)


def main():
    if "--batch" in sys.argv:
        oracle.build()
        batch_fixture()
        return
    quick = "--quick" in sys.argv
    oracle.build()
    with open(os.path.join(HERE, "weights.json"), "w") as f:
        json.dump(weights_fixture(), f)
    with open(os.path.join(HERE, "twiddles.json"), "w") as f:
        json.dump(twiddles_fixture(), f)
    cases = [
        (44497, 2048, 1000), (44497, 2048, 44495),          # config 1: full run, prime
        (86243, 4096, 86241),                               # another Mersenne prime, full run
        (100003, 5184, 3000), (12379, 640, 5000), (1000003, 54432, 2000),
        (2976221, 163840, 5000),                            # config 2 exponent at k
    ]
    cases += [(q, 163840, 5000) for q in composite_draws(3)]  # config 2 composites
    if not quick:
        cases.append((43112609, 2359296, 2000))             # config 3
    entries = []
    path = os.path.join(HERE, "res64.json")
    if os.path.exists(path):
        with open(path) as f:
            entries = json.load(f)
    have = {(e["p"], e["N"], e["k"]) for e in entries}
    for p, N, k in cases:
        if (p, N, k) in have:
            continue
        entries.append(res64_entry(p, N, k))
        with open(path, "w") as f:
            json.dump(entries, f, indent=1)


if __name__ == "__main__":
    main()
