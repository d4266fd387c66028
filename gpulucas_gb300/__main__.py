"""Command line with the reference's flags (gpuLucas.cu:374-454):

    python -m gpulucas_gb300 [-h] [-v] [-q] [-f N] [-n p] [-d dev] [-c freq] [-k iters] [-m fused|plain]
                             [-H h] [-I mode] [-R radix] [-P mode] [p]

-f N    FFT length (even, N/2 = 2^a 3^b 5^c 7^d); without -f the length is chosen as
        findSignalSize does (gpuLucas.cu:1064-1187)
-n p    exponent (or give p as the positional argument)
-d dev  CUDA device
-c freq checkpoint every freq iterations to <p>.chk in the reference's format
        (gpuLucas.cu:1414-1423); a run finding <p>.chk or <p>.chk.bak resumes from it
-k k    stop after k iterations and print Res64 (0 = full p-2 test)
-m      execution form: fused (default) or plain
-H h    fused form: FFT column length h (M = h x w), instead of the timed layout search
-I mode fused form, with -H: column passes 1 in place, 2 in place + prefetched weights,
        3 two columns per CTA, 4 two columns per CTA forward + prefetched weights inverse,
        -1 two-buffer (the layout search picks among these otherwise)
-R r    fused form, with -H: largest radix of the row DFTs (8, 4 or 2)
-P mode fused form, with -H: row pass compiled for any radix (-1), or for radices 4, 3, 2
        only with its stage values in shared memory (1) or read through L1 (2)
SIGINT / SIGTERM write a checkpoint and exit (gpuLucas.cu:365-369, 1425-1429).
A full test appends the reference's result line to results.txt (gpuLucas.cu:1514-1548)
and removes its checkpoint files (gpuLucas.cu:628-632).
"""
from __future__ import annotations

import argparse
import os
import signal
import sys
import time

_stop = False


def _on_signal(sig, frame):
    global _stop
    _stop = True


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="gpulucas_gb300", add_help=False)
    ap.add_argument("-h", action="store_true")
    ap.add_argument("-v", action="store_true")
    ap.add_argument("-q", action="store_true")
    ap.add_argument("-f", type=int, default=0)
    ap.add_argument("-n", type=int, default=0)
    ap.add_argument("-d", type=int, default=0)
    ap.add_argument("-c", type=int, default=0)
    ap.add_argument("-k", type=int, default=0)
    ap.add_argument("-m", choices=["fused", "plain"], default="fused")
    ap.add_argument("-H", type=int, default=0)
    ap.add_argument("-I", type=int, default=0, choices=[-1, 0, 1, 2, 3, 4])
    ap.add_argument("-R", type=int, default=0, choices=[0, 2, 4, 8])
    ap.add_argument("-P", type=int, default=0, choices=[-1, 0, 1, 2])
    ap.add_argument("p", nargs="?", type=int, default=0)
    a = ap.parse_args(argv)
    if a.h:
        print(__doc__, file=sys.stderr)
        return 1
    p = a.n or a.p
    if not p:
        print("testPrime not specified, aborting", file=sys.stderr)
        return 2
    import gpulucas_gb300 as gl
    mode = gl.MODE_FUSED if a.m == "fused" else gl.MODE_PLAIN
    chk = f"{p}.chk"
    resume_k = None
    N = a.f
    if os.path.exists(chk) or os.path.exists(chk + ".bak"):
        try:
            Nc, resume_k, _ = gl.checkpoint_read(chk, p, with_digits=False)
            if N and N != Nc:
                print(f"checkpoint {chk} has N = {Nc}, not {N}; not resuming", file=sys.stderr)
                resume_k = None
            else:
                N = Nc
        except gl.GLError as e:
            print(f"ignoring checkpoint: {e}", file=sys.stderr)
            resume_k = None
    if not N:
        N, ms, err = gl.find_signal_size(p, device=a.d)
        if not a.q:
            print(f"Optimal signalSize detected: {N} ({ms:.4f} ms/iter, trial round-off {err:.4f})")
    total = a.k if a.k else p - 2
    signal.signal(signal.SIGINT, _on_signal)
    signal.signal(signal.SIGTERM, _on_signal)
    t0 = time.time()
    with gl.Plan(p, N, mode=mode, device=a.d, fft_h=a.H, col_inplace=a.I, max_radix_row=a.R,
                 row_pass=a.P) as pl:
        i = pl.info
        if resume_k is not None:
            pl.resume(chk)
            done = resume_k
            if not a.q:
                print(f"Resuming M{p} at iteration {done} from {chk}")
        else:
            pl.reset()
            done = 0
        if not a.q:
            rw = "x".join(str(r) for r in i.radix_w if r)
            rh = "x".join(str(r) for r in i.radix_h if r)
            print(f"Testing M{p}, word sizes ({i.lo_bits}, {i.hi_bits}), FFT length {N} "
                  f"({i.fft_h} x {i.fft_w} complex, columns {rh}, rows {rw}, column passes -I {i.col_variant}, "
                  f"row pass -P {i.row_variant}), "
                  f"carry depth {i.carry_depth}, form {a.m}")
        step = a.c if a.c > 0 else max(1, total - done)
        ms_total, maxerr = 0.0, 0.0
        while done < total and not _stop:
            n = min(step, total - done)
            rep = pl.iterate(n)
            done += n
            ms_total += rep.ms
            maxerr = max(maxerr, rep.max_roundoff)
            if a.c > 0 and (done < total or _stop):
                pl.checkpoint_write(chk)
                if a.v:
                    print(f"[{100.0 * done / total:4.1f}%] Iter {done}: {rep.ms / n:.4f} ms/iter, "
                          f"0x{pl.res64():016x}")
        if _stop and done < total:
            pl.checkpoint_write(chk)
            print(f"Interrupted at iteration {done}; checkpoint written to {chk}")
            return 130
        _, r, z = pl.residue()
    dt = time.time() - t0
    if a.k:
        print(f"M( {p} ) Iter {done}: 0x{r:016x}, max round-off {maxerr:.4f}, "
              f"{ms_total / max(1, done - (resume_k or 0)):.4f} ms/iter, n = {N}")
        return 0
    line = f"M( {p} )P, n = {N}, gpulucas_gb300" if z else f"M( {p} )C, 0x{r:016x}, n = {N}, gpulucas_gb300"
    print(line)
    if a.v:
        print(f"max round-off {maxerr:.4f}, {dt:.1f} s")
    with open("results.txt", "a") as f:
        f.write(line + "\n")
    for path in (chk, chk + ".bak"):
        if os.path.exists(path):
            os.remove(path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
