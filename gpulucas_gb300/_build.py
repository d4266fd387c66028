"""Build libgpulucas_gb300.so in-tree with nvcc for sm_103a (no torch extension machinery).

The translation units compile in parallel; the result lands beside this file and is
what ``gpulucas_gb300`` loads.  Host code is compiled with -ffp-contract=off so the
double-double tables are bit-identical on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgpulucas_gb300.so")
HOSTCHECK = os.path.join(HERE, "libgl_hostcheck.so")
CLI = os.path.join(HERE, "gpulucas")

SOURCES = ["gl_kernels.cu", "gl_residue.cu", "gl_capi.cpp", "gl_tables.cpp", "gl_noalloc.cu", "gl_checkpoint.cpp", "gl_server.cpp",
           "gl_batch.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def common_flags() -> list[str]:
    # every nvcc warning is an error: a host function reached from device code (for
    # instance a plain constexpr helper) compiles to undefined device behaviour
    return ["-O3", "-std=c++17", "-lineinfo", "-Werror", "all-warnings", "-Xcompiler",
            "-fPIC,-ffp-contract=off,-Wall,-Wno-unknown-pragmas", "-I", os.path.join(HERE, "..", "include")] + ARCH


def _check_ptxas(src: str, report: str) -> None:
    """Every kernel must keep its arrays in registers: a stack frame or a spill means a
    dynamically indexed array or register overflow, both a large slowdown."""
    bad = []
    func = None
    for line in report.splitlines():
        if "Compiling entry function" in line or "Function properties for" in line:
            func = line.split("'")[1] if "'" in line else line.split()[-1]
        if "bytes stack frame" in line:
            parts = line.split()
            stack, spill_st, spill_ld = int(parts[0]), int(parts[4]), int(parts[8])
            if stack or spill_st or spill_ld:
                bad.append(f"{func}: {line.strip()}")
    if bad:
        raise RuntimeError(f"{src}: kernels use local memory:\n" + "\n".join(bad))


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + common_flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd = [nvcc(), "-x", "cu"] + common_flags() + ["-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if src.endswith(".cu"):
        _check_ptxas(src, r.stderr)
        if verbose_ptxas:
            sys.stderr.write(r.stderr)
    return obj


def build(verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


def build_cli() -> str:
    """The `gpulucas` executable (the reference's command line) linked to the library."""
    tmp = CLI + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(HERE, "..", "include"),
           os.path.join(CSRC, "gl_cli.cpp"), "-o", tmp, "-L", HERE, "-lgpulucas_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cli build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build_hostcheck() -> str:
    """Host-only build of the device arithmetic helpers, for the CPU test suite."""
    os.makedirs(BUILD, exist_ok=True)
    tmp = HOSTCHECK + ".tmp"
    cmd = [nvcc(), "-x", "cu", "-O2", "-std=c++17", "-shared", "-Werror", "all-warnings", "-Xcompiler",
           "-fPIC,-ffp-contract=off,-Wno-unknown-pragmas",
           os.path.join(CSRC, "gl_hostcheck.cu"), os.path.join(CSRC, "gl_tables.cpp"), "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"hostcheck build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, HOSTCHECK)
    return HOSTCHECK


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
    print(build_hostcheck())
