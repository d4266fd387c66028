"""Seeded synthetic workloads of the batched and served configurations.

Both draw prime exponents; primes come from a numpy sieve (batch range) or a
deterministic Miller-Rabin test (serving range up to 5e7), so nothing beyond numpy
is needed.  The reference has no such workloads (it runs one test per process).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def primes_between(lo: int, hi: int) -> np.ndarray:
    """All primes in [lo, hi] (sieve of Eratosthenes)."""
    sieve = np.ones(hi + 1, dtype=bool)
    sieve[:2] = False
    for i in range(2, int(hi ** 0.5) + 1):
        if sieve[i]:
            sieve[i * i::i] = False
    return np.nonzero(sieve[lo:])[0] + lo


def is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 3.3e24."""
    if n < 2:
        return False
    small = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41)
    for q in small:
        if n % q == 0:
            return n == q
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in small:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def next_prime(n: int) -> int:
    n = max(2, int(n))
    while not is_prime(n):
        n += 1
    return n


def batch_exponents(count: int = 256, lo: int = 100_000, hi: int = 3_000_000, seed: int = 4) -> list[int]:
    """The batched configuration: `count` primes drawn uniformly (without replacement)
    from the primes in [lo, hi] by numpy.random.default_rng(seed)."""
    ps = primes_between(lo, hi)
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.choice(ps, size=count, replace=False)]


@dataclass(frozen=True)
class Request:
    rid: int
    arrival_s: float
    p: int
    iterations: int   # k for a Res64 check, p - 2 for a full test
    full: bool


def serving_requests(count: int, rate_per_s: float = 50.0, seed: int = 5, lo: float = 1e5, hi: float = 5e7,
                     full_fraction: float = 0.2, full_hi: float = 2e6, k: int = 5000) -> list[Request]:
    """The served configuration: Poisson arrivals (mean `rate_per_s`), exponents
    log-uniform in [lo, hi] rounded up to the next prime; a `full_fraction` of the
    requests are full tests with exponents log-uniform in [lo, full_hi], the rest
    Res64 checks after k iterations.  The first `count` arrivals form the window."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += float(rng.exponential(1.0 / rate_per_s))
        full = bool(rng.random() < full_fraction)
        top = full_hi if full else hi
        x = math.exp(float(rng.uniform(math.log(lo), math.log(top))))
        p = next_prime(int(x))
        out.append(Request(rid, t, p, p - 2 if full else k, full))
    return out
