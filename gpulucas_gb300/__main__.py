"""Command line with the reference's flags (gpuLucas.cu:374-454):

    python -m gpulucas_gb300 [-h] [-v] [-q] [-f N] [-n p] [-d dev] [-c freq] [-k iters] [-m fused|plain] [p]

-f N    FFT length (the reference requires N % 256 == 0; here N must be even with
        N/2 = 2^a 3^b 5^c 7^d)
-n p    exponent (or give p as the positional argument)
-d dev  CUDA device
-c freq round-off status check interval in iterations
-k k    stop after k iterations and print Res64 (0 = full p-2 test)
-m      execution form: fused (default) or plain
A full test appends the reference's result line to results.txt (gpuLucas.cu:1514-1548).
"""
from __future__ import annotations

import argparse
import sys
import time


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="gpulucas_gb300", add_help=False)
    ap.add_argument("-h", action="store_true")
    ap.add_argument("-v", action="store_true")
    ap.add_argument("-q", action="store_true")
    ap.add_argument("-f", type=int, default=0)
    ap.add_argument("-n", type=int, default=0)
    ap.add_argument("-d", type=int, default=0)
    ap.add_argument("-c", type=int, default=1000)
    ap.add_argument("-k", type=int, default=0)
    ap.add_argument("-m", choices=["fused", "plain"], default="fused")
    ap.add_argument("p", nargs="?", type=int, default=0)
    a = ap.parse_args(argv)
    if a.h:
        print(__doc__, file=sys.stderr)
        return 1
    p = a.n or a.p
    if not p:
        print("testPrime not specified, aborting", file=sys.stderr)
        return 2
    if not a.f:
        print("an FFT length -f N is required", file=sys.stderr)
        return 2
    import gpulucas_gb300 as gl
    mode = gl.MODE_FUSED if a.m == "fused" else gl.MODE_PLAIN
    t0 = time.time()
    with gl.Plan(p, a.f, mode=mode, device=a.d, check_every=max(1, a.c)) as pl:
        if not a.q:
            i = pl.info
            print(f"Testing M{p}, word sizes ({i.lo_bits}, {i.hi_bits}), FFT length {a.f} "
                  f"({i.fft_h} x {i.fft_w} complex), carry depth {i.carry_depth}, form {a.m}")
        res = pl.mersenne_test(a.k)
    dt = time.time() - t0
    if a.k:
        print(f"M( {p} ) Iter {res.iterations}: 0x{res.res64:016x}, max round-off {res.max_roundoff:.4f}, "
              f"{res.ms / max(1, res.iterations):.4f} ms/iter, n = {a.f}")
        return 0
    line = (f"M( {p} )P, n = {a.f}, gpulucas_gb300" if res.is_prime
            else f"M( {p} )C, 0x{res.res64:016x}, n = {a.f}, gpulucas_gb300")
    print(line)
    if a.v:
        print(f"max round-off {res.max_roundoff:.4f}, {dt:.1f} s")
    with open("results.txt", "a") as f:
        f.write(line + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
