"""The oracle: CPU restatements of the gpuLucas Lucas-Lehmer path, used as the checker.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference legs of ``bench.py`` may import this package.  The product
library (``gpulucas_gb300``) never imports, links or calls anything here.

Three independent implementations:

* ``IBDWT`` -- ``ibdwt_oracle.c``: the reference's irrational-base DWT iteration
  (gpuLucas.cu:845-942 mersenneIter; IrrBaseBalanced.cu:52-169 dicing and final carry;
  gpuLucas.cu:1288-1352 residue), with its own double-double weights and own FFT.
* ``Exact`` -- ``exact_oracle.c``: exact S^2 - 2 mod 2^p - 1 by a number-theoretic
  transform, no floating point.
* ``lucas_lehmer_int`` -- pure Python integers, for small p.

Beside them, ``refrun`` runs the reference program itself (gpuLucas.cu with cuFFT,
compiled for the GPU by ``build_ref.py`` into the git-ignored ``oracle/_ref/``) and reads
its Res64, timings and checkpointed state.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-C", _HERE, "-s"], check=True)
    return _LIB_PATH


def build_ref(force: bool = False):
    """Stage and compile the reference gpuLucas program (oracle/build_ref.py); returns its
    path, or None when neither the reference checkout nor a staged copy is present."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gl_oracle_build_ref", os.path.join(_HERE, "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        sig = {
            "orc_slice_depth": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
            "orc_bits": (None, [ctypes.c_int, ctypes.c_int, i32p, u8p]),
            "orc_bits_refdouble": (None, [ctypes.c_int, ctypes.c_int, i32p]),
            "orc_weights": (None, [ctypes.c_int, ctypes.c_int, f64p, f64p]),
            "orc_twiddles": (None, [ctypes.c_int, f64p, f64p]),
            "orc_create": (P, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "orc_destroy": (None, [P]),
            "orc_reset": (None, [P]),
            "orc_iterate": (None, [P, ctypes.c_int64]),
            "orc_maxerr": (ctypes.c_double, [P]),
            "orc_max_abs_product": (ctypes.c_int64, [P]),
            "orc_overflow": (ctypes.c_int, [P]),
            "orc_iters_done": (ctypes.c_int64, [P]),
            "orc_get_ll": (None, [P, i64p]),
            "orc_get_state": (None, [P, i32p, i8p]),
            "orc_get_signal": (None, [P, f64p]),
            "orc_set_state": (None, [P, i32p, i8p, ctypes.c_int64]),
            "orc_dice": (None, [ctypes.c_int, ctypes.c_int, i64p, i32p, i8p]),
            "orc_rebalance": (None, [ctypes.c_int, ctypes.c_int, i32p, i8p, i32p]),
            "orc_res64_normalize": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int, i32p]),
            "orc_residue": (None, [P, i32p, ctypes.POINTER(ctypes.c_uint64),
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
            "orc_threads": (ctypes.c_int, []),
            "orc_set_threads": (None, [ctypes.c_int]),
            "ex_create": (P, [ctypes.c_int, ctypes.c_int]),
            "ex_destroy": (None, [P]),
            "ex_iterate": (None, [P, ctypes.c_int64]),
            "ex_iters_done": (ctypes.c_int64, [P]),
            "ex_res64": (ctypes.c_uint64, [P]),
            "ex_is_zero": (ctypes.c_int, [P]),
            "ex_words": (ctypes.c_int, [P]),
            "ex_get": (None, [P, u64p]),
            "ex_set": (None, [P, u64p, ctypes.c_int64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


# --------------------------------------------------------------------------- params

def slice_depth(p: int, N: int) -> int:
    """setSliceAndDice (gpuLucas.cu:323-343), table extended to ratio 21; -1 if refused."""
    return lib().orc_slice_depth(p, N)


def bits(p: int, N: int):
    b = np.empty(N, np.int32)
    f = np.empty(N, np.uint8)
    lib().orc_bits(p, N, b, f)
    return b, f


def bits_refdouble(p: int, N: int):
    b = np.empty(N, np.int32)
    lib().orc_bits_refdouble(p, N, b)
    return b


def weights(p: int, N: int):
    """A[j], Ainv[j] = (1/A[j])/N as in computeWeightVectors (gpuLucas.cu:673-686)."""
    A = np.empty(N, np.float64)
    Ai = np.empty(N, np.float64)
    lib().orc_weights(p, N, A, Ai)
    return A, Ai


def twiddles(L: int):
    re = np.empty(L, np.float64)
    im = np.empty(L, np.float64)
    lib().orc_twiddles(L, re, im)
    return re + 1j * im


def dice(p: int, N: int, ll: np.ndarray):
    """llintToIrrBal<n> (IrrBaseBalanced.cu:52-110) over int64 products."""
    ll = np.ascontiguousarray(ll, np.int64)
    d = np.empty(N, np.int32)
    h = np.empty(N, np.int8)
    lib().orc_dice(p, N, ll, d, h)
    return d, h


def rebalance(p: int, N: int, digit: np.ndarray, hi: np.ndarray) -> np.ndarray:
    out = np.empty(N, np.int32)
    lib().orc_rebalance(p, N, np.ascontiguousarray(digit, np.int32),
                        np.ascontiguousarray(hi, np.int8), out)
    return out


def res64_normalize(p: int, N: int, digits: np.ndarray) -> int:
    """print_residue (gpuLucas.cu:1288-1352) on balanced digits (copied, not modified)."""
    d = np.array(digits, np.int32, copy=True)
    return int(lib().orc_res64_normalize(p, N, d))


def digits_to_int(p: int, N: int, digits: np.ndarray) -> int:
    """Exact value of a balanced variable-base digit vector mod 2^p - 1."""
    b, _ = bits(p, N)
    M = (1 << p) - 1
    v = 0
    pos = 0
    for j in range(N):
        v += int(digits[j]) << pos
        pos += int(b[j])
    return v % M


def carry_state_to_int(p: int, N: int, digit: np.ndarray, hi: np.ndarray) -> int:
    """Value of a carry-save state (digit[j] + hi[j-1]) mod 2^p - 1."""
    d = digit.astype(np.int64) + np.roll(hi.astype(np.int64), 1)
    return digits_to_int(p, N, d)


# --------------------------------------------------------------------------- IBDWT

class IBDWT:
    """The reference's IBDWT Lucas-Lehmer iteration on the CPU (ibdwt_oracle.c)."""

    def __init__(self, p: int, N: int, threads: int = 0):
        self.p, self.N = p, N
        self._L = lib()
        self._c = self._L.orc_create(p, N, threads)
        if not self._c:
            raise ValueError(f"oracle refuses p={p} N={N}")
        self._L.orc_reset(self._c)

    def close(self):
        if self._c:
            self._L.orc_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        self._L.orc_reset(self._c)

    def iterate(self, k: int):
        self._L.orc_iterate(self._c, int(k))
        return self

    @property
    def iters_done(self) -> int:
        return int(self._L.orc_iters_done(self._c))

    @property
    def maxerr(self) -> float:
        return float(self._L.orc_maxerr(self._c))

    @property
    def max_abs_product(self) -> int:
        return int(self._L.orc_max_abs_product(self._c))

    @property
    def overflow(self) -> bool:
        return bool(self._L.orc_overflow(self._c))

    def ll(self) -> np.ndarray:
        out = np.empty(self.N, np.int64)
        self._L.orc_get_ll(self._c, out)
        return out

    def state(self):
        d = np.empty(self.N, np.int32)
        h = np.empty(self.N, np.int8)
        self._L.orc_get_state(self._c, d, h)
        return d, h

    def signal(self) -> np.ndarray:
        out = np.empty(self.N, np.float64)
        self._L.orc_get_signal(self._c, out)
        return out

    def set_state(self, digit, hi, iters_done: int):
        self._L.orc_set_state(self._c, np.ascontiguousarray(digit, np.int32),
                              np.ascontiguousarray(hi, np.int8), int(iters_done))

    def residue(self):
        """(rebalanced digits, res64, reference zero test, exact zero test)."""
        d = np.empty(self.N, np.int32)
        r = ctypes.c_uint64()
        rz = ctypes.c_int()
        ez = ctypes.c_int()
        self._L.orc_residue(self._c, d, ctypes.byref(r), ctypes.byref(rz), ctypes.byref(ez))
        return d, int(r.value), bool(rz.value), bool(ez.value)

    def res64(self) -> int:
        return self.residue()[1]


# --------------------------------------------------------------------------- exact

class Exact:
    """Exact S_k mod 2^p - 1 by NTT squaring (exact_oracle.c)."""

    def __init__(self, p: int, threads: int = 0):
        self.p = p
        self._L = lib()
        self._c = self._L.ex_create(p, threads)
        if not self._c:
            raise ValueError(f"exact oracle refuses p={p}")

    def close(self):
        if self._c:
            self._L.ex_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def iterate(self, k: int):
        self._L.ex_iterate(self._c, int(k))
        return self

    @property
    def iters_done(self) -> int:
        return int(self._L.ex_iters_done(self._c))

    def res64(self) -> int:
        return int(self._L.ex_res64(self._c))

    def is_zero(self) -> bool:
        return bool(self._L.ex_is_zero(self._c))

    def value(self) -> int:
        w = self._L.ex_words(self._c)
        out = np.empty(w, np.uint64)
        self._L.ex_get(self._c, out)
        return int.from_bytes(out.tobytes(), "little")


def lucas_lehmer_int(p: int, k: int) -> int:
    """S_k mod 2^p - 1 with Python integers (S_0 = 4)."""
    M = (1 << p) - 1
    s = 4
    for _ in range(k):
        s = (s * s - 2) % M
    return s


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def threads() -> int:
    return int(lib().orc_threads())
