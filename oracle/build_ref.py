"""Recipe: build the reference gpuLucas program (cuFFT path) for sm_103a, as an oracle.

TEST INFRASTRUCTURE ONLY.  The program this makes is run by the GPU tests (Res64 and
checkpointed state compared with this project's library) and by bench.py's baseline leg
(the reference's iteration rate on the same GPU).  The product library never links,
loads or runs it.

Two steps, both writing only under ``oracle/_ref/`` (git-ignored, so the reference's
sources never enter this repository's history):

1. stage -- where a checkout of the reference is present (``GL_REFERENCE_DIR``, default
   ``/root/reference``), copy its three sources ``gpuLucas.cu``, ``IrrBaseBalanced.cu``
   and ``cuda_safecalls.h`` into ``oracle/_ref/src/``, applying the patches listed in
   ``PATCHES`` below.  The staged copy travels with the working tree to machines that
   have no reference checkout (the GPU machines), where step 2 runs on it.
2. compile -- ``nvcc`` on the staged ``gpuLucas.cu`` (it includes the other two) with the
   reference Makefile's flags (``-O3 -use_fast_math``, host ``-O3 -fno-strict-aliasing``;
   Makefile:9-11) but ``-gencode arch=compute_103a,code=sm_103a`` in place of its
   compute_20 / compute_13 targets (Makefile:4, rejected by CUDA 13), host
   ``-ffp-contract=off``, and ``-I oracle/ref_shim`` for ``qd/dd_real.h`` (this
   project's own double-double stand-in for the absent QD library); linked with
   ``-lcufft`` (gpuLucas.cu:996-997) instead of ``-lqd``.  Output: ``oracle/_ref/gpuLucas``.

The patches change no arithmetic.  Each removes a hazard for a shared GPU or a compile
error on CUDA 13; ``PATCHES`` gives the reason for each.

Usage: ``python oracle/build_ref.py [--force]``; ``oracle.build_ref()`` calls the same.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(REF_OUT, "src")
BINARY = os.path.join(REF_OUT, "gpuLucas")
SHIM = os.path.join(HERE, "ref_shim")
SOURCES = ("gpuLucas.cu", "IrrBaseBalanced.cu", "cuda_safecalls.h")

# (file, reference lines, old text, new text, reason).  Every old text must occur in the
# reference exactly once.
PATCHES = [
    ("cuda_safecalls.h", "159",
     "int compute_perf  = deviceProp.multiProcessorCount * sm_per_multiproc * deviceProp.clockRate;",
     "int compute_perf  = deviceProp.multiProcessorCount * sm_per_multiproc;",
     "cudaDeviceProp::clockRate no longer exists in CUDA 13; the function "
     "(cutGetMaxGflopsDeviceId) is never called"),
    ("gpuLucas.cu", "738",
     "ival[i] = i_hiBitArr[tid  + i*blockDim.x -1];",
     "ival[i] = (tid + i*blockDim.x > 0) ? i_hiBitArr[tid + i*blockDim.x - 1] : 0;",
     "loadIntToDoubleIBDWT read i_hiBitArr[-1] (one byte before the allocation) in "
     "thread 0; that value is overwritten at gpuLucas.cu:742, so the guard changes no "
     "result"),
    ("gpuLucas.cu", "654",
     "\t\ttemp[i] = z_signal[tid + i*blockDim.x];\n",
     "\t\tif (tid + i*blockDim.x < size) temp[i] = z_signal[tid + i*blockDim.x];\n",
     "ComplexPointwiseSqr loaded up to 255 elements past the N/2+1 spectrum before its "
     "bounds check (the grid is rounded up); those values were never used"),
    ("gpuLucas.cu", "965",
     "if ((unsigned int)free_mem/1024 < estimated_size) {\n\t\t// We don't",
     "if ((size_t)free_mem/1024 < estimated_size) {\n\t\t// We don't",
     "the free-memory check truncated size_t to 32 bits; on a GPU with more than 4 GiB "
     "free it could report too little memory, and errorTrial (gpuLucas.cu:1198) ignores "
     "the failure and launches its kernels on unallocated arrays"),
    ("gpuLucas.cu", "968",
     "if ((unsigned int)free_mem/1024 < estimated_size) {\n\t\t\tprintf",
     "if ((size_t)free_mem/1024 < estimated_size) {\n\t\t\tprintf",
     "same truncation in the in-place fallback's check"),
]


def reference_dir() -> str:
    return os.environ.get("GL_REFERENCE_DIR", "/root/reference")


def _sha256(path: str) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def stage(ref: str | None = None) -> bool:
    """Copy and patch the reference sources into oracle/_ref/src.  False when the
    reference checkout is absent (the staged copy, if any, is kept)."""
    ref = ref or reference_dir()
    if not all(os.path.isfile(os.path.join(ref, s)) for s in SOURCES):
        return False
    texts = {}
    for s in SOURCES:
        with open(os.path.join(ref, s), "r", encoding="latin-1") as f:
            texts[s] = f.read()
    for fname, lines, old, new, why in PATCHES:
        n = texts[fname].count(old)
        if n != 1:
            raise RuntimeError(f"patch for {fname}:{lines} matches {n} times (expected 1): {why}")
        texts[fname] = texts[fname].replace(old, new)
    tmp = SRC_DIR + ".tmp"
    if os.path.isdir(tmp):
        shutil.rmtree(tmp)
    os.makedirs(tmp)
    for s in SOURCES:
        with open(os.path.join(tmp, s), "w", encoding="latin-1") as f:
            f.write(texts[s])
    with open(os.path.join(tmp, "PROVENANCE"), "w") as f:
        f.write(f"staged from {ref}\n")
        for s in SOURCES:
            f.write(f"sha256 {s} {_sha256(os.path.join(ref, s))}\n")
        for fname, lines, _, _, why in PATCHES:
            f.write(f"patch {fname}:{lines}: {why}\n")
    if os.path.isdir(SRC_DIR):
        shutil.rmtree(SRC_DIR)
    os.replace(tmp, SRC_DIR)
    return True


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def compile_staged() -> str:
    src = os.path.join(SRC_DIR, "gpuLucas.cu")
    if not os.path.isfile(src):
        raise FileNotFoundError("no staged reference sources under oracle/_ref/src")
    tmp = BINARY + ".tmp"
    cmd = [nvcc(), "-O3", "-use_fast_math", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", SHIM, "-Xcompiler", "-O3,-fno-strict-aliasing,-ffp-contract=off",
           "-o", tmp, src, "-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, BINARY)
    return BINARY


def build(force: bool = False) -> str | None:
    """Stage (where the reference is present) and compile.  Returns the binary's path, or
    None when neither the reference nor a staged copy is available."""
    staged = stage()
    if not os.path.isfile(os.path.join(SRC_DIR, "gpuLucas.cu")):
        return None
    if force or staged or not os.path.isfile(BINARY):
        return compile_staged()
    return BINARY


if __name__ == "__main__":
    out = build(force="--force" in sys.argv)
    print(out if out else "reference sources unavailable: nothing built")
