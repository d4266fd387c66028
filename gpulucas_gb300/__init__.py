"""gpulucas_gb300 -- GB300-native Lucas-Lehmer engine (IBDWT, FP64, sm_103a kernels).

Python mirror of the reference's entry points over the C ABI (include/gpulucas.h):

* ``mersenneTest(p, N)``  -- full test (gpuLucas.cu:1358-1551, README errorTest/mersenneTest)
* ``errorTest(p, N)``     -- timing/round-off trial (errorTrial, gpuLucas.cu:1192-1282)
* ``setSliceAndDice(p, N)`` -- carry depth n of llintToIrrBal<n> (gpuLucas.cu:323-343)
* ``Plan``               -- a per-test plan: iterate, products, carry state, residue

All compute runs in ``libgpulucas_gb300.so``; there is no CPU fallback.  Importing this
package without the built library raises ImportError (run ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgpulucas_gb300.so")

GL_OK = 0
GL_ERR_ARG = -1
GL_ERR_RATIO = -2
GL_ERR_SIZE = -3
GL_ERR_CUDA = -4
GL_ERR_NOMEM = -5
GL_ERR_ROUNDOFF = -6
GL_ERR_OVERFLOW = -7
GL_ERR_NODEVICE = -8
GL_ERR_IO = -9
GL_ERR_CHECKPOINT = -10
GL_ERR_STATE = -11
GL_ERR_TOO_LARGE = -12
GL_ERR_TIMEOUT = -13
NOALLOC_MAX_N = 65536

MODE_FUSED = 0
MODE_PLAIN = 1


class PlanOpts(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("device", ctypes.c_int), ("error_limit", ctypes.c_double),
                ("check_every", ctypes.c_int), ("use_graphs", ctypes.c_int), ("fft_h", ctypes.c_int),
                ("cols_per_cta", ctypes.c_int), ("autotune", ctypes.c_int), ("batch_layout", ctypes.c_int),
                ("high_priority", ctypes.c_int), ("max_radix_col", ctypes.c_int),
                ("max_radix_row", ctypes.c_int), ("resident", ctypes.c_int),
                ("col_inplace", ctypes.c_int), ("row_pass", ctypes.c_int)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("p", ctypes.c_int), ("N", ctypes.c_int), ("lo_bits", ctypes.c_int), ("hi_bits", ctypes.c_int),
                ("carry_depth", ctypes.c_int), ("mode", ctypes.c_int), ("fft_w", ctypes.c_int),
                ("fft_h", ctypes.c_int), ("cols_per_cta", ctypes.c_int), ("radix_w", ctypes.c_int * 8),
                ("radix_h", ctypes.c_int * 8), ("threads_col", ctypes.c_int), ("threads_row", ctypes.c_int),
                ("smem_col", ctypes.c_int), ("smem_row", ctypes.c_int), ("device_bytes", ctypes.c_size_t),
                ("resident_ctas", ctypes.c_int), ("resident_smem", ctypes.c_int), ("col_variant", ctypes.c_int),
                ("row_variant", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("ntests", ctypes.c_int), ("col_units", ctypes.c_int), ("row_units", ctypes.c_int),
                ("threads_col", ctypes.c_int), ("threads_row", ctypes.c_int), ("smem_col", ctypes.c_int),
                ("smem_row", ctypes.c_int), ("device_bytes", ctypes.c_size_t), ("iterations", ctypes.c_int64)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_double), ("max_active", ctypes.c_int),
                ("step_ms", ctypes.c_double), ("checkpoint_every", ctypes.c_int64),
                ("max_bits_per_word", ctypes.c_double), ("retries", ctypes.c_int),
                ("chain_iterations", ctypes.c_int64), ("lanes", ctypes.c_int), ("build_threads", ctypes.c_int),
                ("error_limit", ctypes.c_double), ("check_every", ctypes.c_int), ("reserved", ctypes.c_int * 8)]


class Completion(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("p", ctypes.c_int), ("N", ctypes.c_int), ("iterations", ctypes.c_int64),
                ("full", ctypes.c_int), ("status", ctypes.c_int), ("is_zero", ctypes.c_int),
                ("is_prime", ctypes.c_int), ("res64", ctypes.c_uint64), ("max_roundoff", ctypes.c_double),
                ("arrival_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("attempts", ctypes.c_int), ("lane", ctypes.c_int), ("n_checkpoints", ctypes.c_int),
                ("reserved", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("wall_s", ctypes.c_double), ("lane_busy_s", ctypes.c_double * 3), ("steps", ctypes.c_int64 * 3),
                ("rebuilds", ctypes.c_int64 * 3), ("peak_live", ctypes.c_int * 3), ("live", ctypes.c_int),
                ("queued", ctypes.c_int), ("building", ctypes.c_int), ("bytes_in_use", ctypes.c_size_t),
                ("peak_bytes", ctypes.c_size_t), ("flop_alg", ctypes.c_double), ("submitted", ctypes.c_int64),
                ("completed", ctypes.c_int64)]


# callbacks of gl_server_engine
ENGINE_SIGNAL_SIZE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int))
ENGINE_FOOTPRINT = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_size_t))
ENGINE_CREATE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_void_p))
ENGINE_DESTROY = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)
ENGINE_BATCH = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                ctypes.c_int, ctypes.POINTER(ctypes.c_void_p))
ENGINE_CLOSE_BATCH = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)
ENGINE_START = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64)
ENGINE_READY = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)
ENGINE_FINISH = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int))
ENGINE_RES64 = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                ctypes.POINTER(ctypes.c_int))


class ServerEngine(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("signal_size", ENGINE_SIGNAL_SIZE), ("footprint", ENGINE_FOOTPRINT),
                ("create", ENGINE_CREATE), ("destroy", ENGINE_DESTROY), ("batch", ENGINE_BATCH),
                ("close_batch", ENGINE_CLOSE_BATCH), ("start", ENGINE_START), ("ready", ENGINE_READY),
                ("finish", ENGINE_FINISH), ("res64", ENGINE_RES64)]


class IterReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("total_iterations", ctypes.c_int64),
                ("max_roundoff", ctypes.c_double), ("ms", ctypes.c_double), ("status", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("p", ctypes.c_int), ("N", ctypes.c_int), ("iterations", ctypes.c_int64),
                ("is_prime", ctypes.c_int), ("is_zero", ctypes.c_int), ("res64", ctypes.c_uint64),
                ("max_roundoff", ctypes.c_double), ("ms", ctypes.c_double)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() "
                          "(this package has no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    PP = ctypes.POINTER(ctypes.c_void_p)
    vp = ctypes.c_void_p
    sig = {
        "gl_default_opts": (ctypes.c_int, [ctypes.POINTER(PlanOpts)]),
        "gl_plan_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(PlanOpts), PP]),
        "gl_plan_destroy": (ctypes.c_int, [P]),
        "gl_plan_get_info": (ctypes.c_int, [P, ctypes.POINTER(PlanInfo)]),
        "gl_plan_describe": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(PlanOpts),
                                            ctypes.POINTER(PlanInfo)]),
        "gl_reset": (ctypes.c_int, [P]),
        "gl_iterate": (ctypes.c_int, [P, ctypes.c_int64, ctypes.POINTER(IterReport)]),
        "gl_plan_stream": (ctypes.c_int, [P, PP]),
        "gl_enqueue": (ctypes.c_int, [P, ctypes.c_int64]),
        "gl_sync_status": (ctypes.c_int, [P, ctypes.POINTER(IterReport)]),
        "gl_launches_per_iteration": (ctypes.c_int, [P]),
        "gl_profile_kernels": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_int)]),
        "gl_get_products": (ctypes.c_int, [P, vp]),
        "gl_get_carry_state": (ctypes.c_int, [P, vp, vp]),
        "gl_set_products": (ctypes.c_int, [P, vp, ctypes.c_int64]),
        "gl_set_carry_state": (ctypes.c_int, [P, vp, vp, ctypes.c_int64]),
        "gl_iterate_host": (ctypes.c_int, [P, vp, vp, ctypes.c_int64, vp, vp, ctypes.POINTER(IterReport)]),
        "gl_iterate_host_words": (ctypes.c_int, [P, vp, ctypes.c_int64, vp, ctypes.POINTER(IterReport)]),
        "gl_get_residue": (ctypes.c_int, [P, vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)]),
        "errorTest": (ctypes.c_float, [ctypes.c_int, ctypes.c_int]),
        "mersenneTest": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
        "setSliceAndDice": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
        "gl_error_test": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(PlanOpts), ctypes.c_int,
                                         ctypes.POINTER(IterReport)]),
        "gl_mersenne_test": (ctypes.c_int, [P, ctypes.c_int64, ctypes.POINTER(Result)]),
        "gl_error_string": (ctypes.c_char_p, [ctypes.c_int]),
        "gl_version": (ctypes.c_int, []),
        "gl_probe_fp64_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
        "gl_probe_fp64_butterfly": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
        "gl_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
        "gl_find_signal_size": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(PlanOpts), ctypes.POINTER(ctypes.c_int),
                                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
        "gl_smallest_signal_size": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]),
        "gl_safe_signal_size": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
        "gl_fast_signal_size": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]),
        "gl_batch_create": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.POINTER(PlanOpts), PP]),
        "gl_batch_create_from_plans": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(PlanOpts), PP]),
        "gl_batch_query": (ctypes.c_int, [P]),
        "gl_batch_test_status": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_int)]),
        "gl_batch_destroy": (ctypes.c_int, [P]),
        "gl_batch_iterate": (ctypes.c_int, [P, ctypes.c_int64, ctypes.POINTER(IterReport)]),
        "gl_batch_stream": (ctypes.c_int, [P, PP]),
        "gl_batch_enqueue": (ctypes.c_int, [P, ctypes.c_int64]),
        "gl_batch_sync_status": (ctypes.c_int, [P, ctypes.POINTER(IterReport)]),
        "gl_batch_result": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(Result), ctypes.POINTER(ctypes.c_int)]),
        "gl_batch_get_info": (ctypes.c_int, [P, ctypes.POINTER(BatchInfo)]),
        "gl_batch_test_info": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(PlanInfo)]),
        "gl_checkpoint_write": (ctypes.c_int, [P, ctypes.c_char_p]),
        "gl_checkpoint_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int64), vp]),
        "gl_plan_resume": (ctypes.c_int, [P, ctypes.c_char_p]),
        "gl_server_default_opts": (ctypes.c_int, [ctypes.POINTER(ServerOpts)]),
        "gl_server_create": (ctypes.c_int, [ctypes.POINTER(ServerOpts), ctypes.POINTER(ServerEngine), PP]),
        "gl_server_submit": (ctypes.c_int, [P, ctypes.c_int64, ctypes.c_int, ctypes.c_int64]),
        "gl_server_poll": (ctypes.c_int, [P, ctypes.POINTER(Completion), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                          ctypes.c_double]),
        "gl_server_drain": (ctypes.c_int, [P]),
        "gl_server_checkpoints": (ctypes.c_int, [P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
                                                 ctypes.POINTER(ctypes.c_uint64), ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_int)]),
        "gl_server_get_stats": (ctypes.c_int, [P, ctypes.POINTER(ServerStats)]),
        "gl_server_destroy": (ctypes.c_int, [P]),
        "gl_iterate_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int64,
                                              ctypes.POINTER(ctypes.c_double), vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


lib = _load()

# exported C symbols that include/gpulucas.h declares (checked by the tests)
ABI_SYMBOLS = tuple(sorted([
    "gl_default_opts", "gl_plan_create", "gl_plan_destroy", "gl_plan_get_info", "gl_plan_describe",
    "gl_reset", "gl_iterate",
    "gl_plan_stream", "gl_enqueue", "gl_sync_status", "gl_launches_per_iteration", "gl_profile_kernels",
    "gl_get_products",
    "gl_get_carry_state", "gl_set_products", "gl_set_carry_state", "gl_get_residue", "errorTest",
    "mersenneTest", "setSliceAndDice", "gl_error_test", "gl_mersenne_test", "gl_error_string", "gl_version",
    "gl_probe_fp64_peak", "gl_probe_fp64_butterfly", "gl_iterate_noalloc", "gl_find_signal_size", "gl_checkpoint_write",
    "gl_checkpoint_read", "gl_plan_resume", "gl_smallest_signal_size", "gl_batch_create", "gl_batch_destroy",
    "gl_batch_iterate", "gl_batch_stream", "gl_batch_enqueue", "gl_batch_sync_status", "gl_batch_result",
    "gl_batch_get_info", "gl_batch_test_info", "gl_batch_create_from_plans", "gl_batch_test_status", "gl_safe_signal_size", "gl_batch_query", "gl_fast_signal_size",
    "gl_server_default_opts", "gl_server_create", "gl_server_submit", "gl_server_poll", "gl_server_drain",
    "gl_server_checkpoints", "gl_server_get_stats", "gl_server_destroy", "gl_selftest_bounded_wait",
    "gl_iterate_host", "gl_iterate_host_words",
]))


class GLError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib.gl_error_string(status).decode()
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def _check(status: int, what: str) -> int:
    if status < 0:
        raise GLError(status, what)
    return status


def default_opts(**kw) -> PlanOpts:
    o = PlanOpts()
    lib.gl_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown plan option {k}")
        setattr(o, k, v)
    return o


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class Plan:
    """One Lucas-Lehmer test of 2^p - 1 at FFT length N on one GPU."""

    def __init__(self, p: int, N: int, mode: int = MODE_FUSED, **opts):
        self.p, self.N = int(p), int(N)
        o = default_opts(mode=mode, **opts)
        h = ctypes.c_void_p()
        _check(lib.gl_plan_create(self.p, self.N, ctypes.byref(o), ctypes.byref(h)), f"plan p={p} N={N}")
        self._h = h
        info = PlanInfo()
        _check(lib.gl_plan_get_info(self._h, ctypes.byref(info)), "plan info")
        self.info = info
        self.N = info.N  # N = 0 asks the library to choose it

    # lifetime -----------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib.gl_plan_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # state -------------------------------------------------------------------
    def reset(self):
        _check(lib.gl_reset(self._h), "reset")

    def iterate(self, iters: int, check: bool = True) -> IterReport:
        rep = IterReport()
        st = lib.gl_iterate(self._h, int(iters), ctypes.byref(rep))
        if check:
            _check(st, "iterate")
        return rep

    def enqueue(self, iters: int):
        _check(lib.gl_enqueue(self._h, int(iters)), "enqueue")

    def sync_status(self, check: bool = True) -> IterReport:
        rep = IterReport()
        st = lib.gl_sync_status(self._h, ctypes.byref(rep))
        if check:
            _check(st, "status")
        return rep

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        _check(lib.gl_plan_stream(self._h, ctypes.byref(s)), "stream")
        return s.value or 0

    @property
    def launches_per_iteration(self) -> int:
        return _check(lib.gl_launches_per_iteration(self._h), "launches")

    def profile_kernels(self, iters: int = 10) -> dict:
        """Average ms per launch of each fused kernel (events between launches)."""
        ms = (ctypes.c_double * 3)()
        names = (ctypes.c_char_p * 3)()
        nk = ctypes.c_int()
        _check(lib.gl_profile_kernels(self._h, int(iters), ms, names, ctypes.byref(nk)), "profile_kernels")
        return {names[i].decode(): ms[i] for i in range(nk.value)}

    def products(self) -> np.ndarray:
        out = np.empty(self.N, np.int64)
        _check(lib.gl_get_products(self._h, _ptr(out)), "products")
        return out

    def set_products(self, ll: np.ndarray, iterations: int = 0):
        ll = np.ascontiguousarray(ll, np.int64)
        assert ll.shape == (self.N,)
        _check(lib.gl_set_products(self._h, _ptr(ll), int(iterations)), "set_products")

    def carry_state(self):
        d = np.empty(self.N, np.int32)
        h = np.empty(self.N, np.int8)
        _check(lib.gl_get_carry_state(self._h, _ptr(d), _ptr(h)), "carry_state")
        return d, h

    def iterate_host(self, digit: np.ndarray, hi: np.ndarray, iters: int, check: bool = True):
        """(digit, hi, report): `iters` iterations from a host-held carry-save state."""
        d = np.ascontiguousarray(digit, np.int32)
        h = np.ascontiguousarray(hi, np.int8)
        do = np.empty(self.N, np.int32)
        ho = np.empty(self.N, np.int8)
        rep = IterReport()
        st = lib.gl_iterate_host(self._h, _ptr(d), _ptr(h), int(iters), _ptr(do), _ptr(ho), ctypes.byref(rep))
        if check:
            _check(st, "iterate_host")
        return do, ho, rep

    def iterate_host_words(self, words: np.ndarray, iters: int, check: bool = True):
        """(words, report): `iters` iterations from host-held carry-added words
        (digit[j] + hi[j-1], 4 bytes per word)."""
        w = np.ascontiguousarray(words, np.int32)
        out = np.empty(self.N, np.int32)
        rep = IterReport()
        st = lib.gl_iterate_host_words(self._h, _ptr(w), int(iters), _ptr(out), ctypes.byref(rep))
        if check:
            _check(st, "iterate_host_words")
        return out, rep

    def set_carry_state(self, digit: np.ndarray, hi: np.ndarray, iterations: int):
        d = np.ascontiguousarray(digit, np.int32)
        h = np.ascontiguousarray(hi, np.int8)
        _check(lib.gl_set_carry_state(self._h, _ptr(d), _ptr(h), int(iterations)), "set_carry_state")

    def residue(self):
        """(rebalanced digits, res64, is_zero) of the current state."""
        d = np.empty(self.N, np.int32)
        r = ctypes.c_uint64()
        z = ctypes.c_int()
        _check(lib.gl_get_residue(self._h, _ptr(d), ctypes.byref(r), ctypes.byref(z)), "residue")
        return d, int(r.value), bool(z.value)

    def res64(self) -> int:
        return self.res64_zero()[0]

    def res64_zero(self):
        """(res64, is_zero) of the current state; the digits stay on the device."""
        r = ctypes.c_uint64()
        z = ctypes.c_int()
        _check(lib.gl_get_residue(self._h, None, ctypes.byref(r), ctypes.byref(z)), "residue")
        return int(r.value), bool(z.value)

    def checkpoint_write(self, path: str):
        """Write the state in the reference's <p>.chk format (old file kept as path.bak)."""
        _check(lib.gl_checkpoint_write(self._h, os.fsencode(path)), f"checkpoint_write {path}")

    def resume(self, path: str):
        """Continue from a checkpoint in the reference's format (same p and N)."""
        _check(lib.gl_plan_resume(self._h, os.fsencode(path)), f"resume {path}")

    def mersenne_test(self, iters: int = 0) -> Result:
        res = Result()
        st = lib.gl_mersenne_test(self._h, int(iters), ctypes.byref(res))
        _check(st, "mersenne_test")
        return res


class Batch:
    """Many LL tests advanced together by one set of launches per iteration."""

    def __init__(self, ps=None, Ns=None, *, plans=None, **opts):
        self._plans = None
        if plans is not None:
            # a batch over existing fused-form plans, which it does not own
            plans = list(plans)
            assert plans and ps is None and Ns is None
            arr = (ctypes.c_void_p * len(plans))(*[pl._h.value for pl in plans])
            o = default_opts(**opts)
            h = ctypes.c_void_p()
            _check(lib.gl_batch_create_from_plans(arr, len(plans), ctypes.byref(o), ctypes.byref(h)),
                   f"batch over {len(plans)} plans")
            self._h = h
            self._plans = plans
            self.ntests = len(plans)
            self.info = BatchInfo()
            _check(lib.gl_batch_get_info(self._h, ctypes.byref(self.info)), "batch info")
            return
        ps = np.ascontiguousarray(ps, np.int32)
        Ns = np.zeros_like(ps) if Ns is None else np.ascontiguousarray(Ns, np.int32)
        assert ps.shape == Ns.shape and ps.ndim == 1 and ps.size > 0
        o = default_opts(**opts)
        h = ctypes.c_void_p()
        _check(lib.gl_batch_create(_ptr(ps), _ptr(Ns), int(ps.size), ctypes.byref(o), ctypes.byref(h)),
               f"batch of {ps.size}")
        self._h = h
        self.ntests = int(ps.size)
        self.info = BatchInfo()
        _check(lib.gl_batch_get_info(self._h, ctypes.byref(self.info)), "batch info")

    def close(self):
        if getattr(self, "_h", None):
            lib.gl_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def iterate(self, iters: int, check: bool = True) -> IterReport:
        rep = IterReport()
        st = lib.gl_batch_iterate(self._h, int(iters), ctypes.byref(rep))
        if check:
            _check(st, "batch iterate")
        return rep

    def enqueue(self, iters: int):
        _check(lib.gl_batch_enqueue(self._h, int(iters)), "batch enqueue")

    def query(self) -> bool:
        """True once all enqueued work has finished (does not wait)."""
        return bool(_check(lib.gl_batch_query(self._h), "batch query"))

    def sync_status(self, check: bool = True) -> IterReport:
        rep = IterReport()
        st = lib.gl_batch_sync_status(self._h, ctypes.byref(rep))
        if check:
            _check(st, "batch status")
        return rep

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        _check(lib.gl_batch_stream(self._h, ctypes.byref(s)), "batch stream")
        return s.value or 0

    def test_info(self, i: int) -> PlanInfo:
        info = PlanInfo()
        _check(lib.gl_batch_test_info(self._h, int(i), ctypes.byref(info)), "batch test info")
        return info

    def test_status(self, i: int):
        """(max round-off, status) of test i as of the last status read."""
        e = ctypes.c_double()
        st = ctypes.c_int()
        _check(lib.gl_batch_test_status(self._h, int(i), ctypes.byref(e), ctypes.byref(st)), f"batch status {i}")
        return e.value, st.value

    def result(self, i: int):
        """(Result, status) of test i."""
        r = Result()
        st = ctypes.c_int()
        _check(lib.gl_batch_result(self._h, int(i), ctypes.byref(r), ctypes.byref(st)), f"batch result {i}")
        return r, st.value


def safe_signal_size(p: int) -> int:
    """Smallest length whose word size keeps the measured round-off <= 0.125 (host only)."""
    N = ctypes.c_int()
    _check(lib.gl_safe_signal_size(int(p), ctypes.byref(N)), "safe_signal_size")
    return N.value


def fast_signal_size(p: int, slack: float = 0.2) -> int:
    """Cheapest modelled length within (1 + slack) of safe_signal_size (host only)."""
    N = ctypes.c_int()
    _check(lib.gl_fast_signal_size(int(p), float(slack), ctypes.byref(N)), "fast_signal_size")
    return N.value


def smallest_signal_size(p: int, max_bits_per_word: float = 19.5) -> int:
    N = ctypes.c_int()
    _check(lib.gl_smallest_signal_size(int(p), float(max_bits_per_word), ctypes.byref(N)), "smallest_signal_size")
    return N.value


# reference-named entry points ---------------------------------------------------

def mersenneTest(testPrime: int, signalSize: int) -> int:
    """1 if 2^p - 1 is prime, 0 if composite (prints the reference's result line)."""
    return _check(lib.mersenneTest(int(testPrime), int(signalSize)), "mersenneTest")


def errorTest(testPrime: int, signalSize: int) -> float:
    """Average ms per iteration over clamp(p/10000, 100, 2500) iterations, -1 on error."""
    return float(lib.errorTest(int(testPrime), int(signalSize)))


def setSliceAndDice(testPrime: int, signalSize: int) -> int:
    """Carry depth n of llintToIrrBal<n> for p/N; raises for ratio >= 22."""
    return _check(lib.setSliceAndDice(int(testPrime), int(signalSize)), "setSliceAndDice")


def error_test(p: int, N: int, iters: int = 0, **opts) -> IterReport:
    rep = IterReport()
    o = default_opts(**opts)
    _check(lib.gl_error_test(int(p), int(N), ctypes.byref(o), int(iters), ctypes.byref(rep)), "error_test")
    return rep


def checkpoint_read(path: str, p: int, with_digits: bool = True):
    """(N, squarings done, digits or None) of a checkpoint in the reference's format."""
    N = ctypes.c_int()
    k = ctypes.c_int64()
    _check(lib.gl_checkpoint_read(os.fsencode(path), int(p), ctypes.byref(N), ctypes.byref(k), None),
           f"checkpoint_read {path}")
    digits = None
    if with_digits:
        digits = np.empty(N.value, np.int32)
        _check(lib.gl_checkpoint_read(os.fsencode(path), int(p), ctypes.byref(N), ctypes.byref(k),
                                      _ptr(digits)), f"checkpoint_read {path}")
    return N.value, k.value, digits


def find_signal_size(p: int, **opts):
    """(N, ms per iteration, max round-off of the trial) chosen for exponent p."""
    N = ctypes.c_int()
    ms = ctypes.c_double()
    err = ctypes.c_double()
    o = default_opts(**opts)
    _check(lib.gl_find_signal_size(int(p), ctypes.byref(o), ctypes.byref(N), ctypes.byref(ms), ctypes.byref(err)),
           f"find_signal_size p={p}")
    return N.value, ms.value, err.value


def iterate_noalloc(p: int, N: int, ll_in_ptr: int, ll_out_ptr: int, iters: int, stream: int = 0) -> float:
    """LL iterations on caller-owned device products without any device allocation
    (see gl_iterate_noalloc in include/gpulucas.h); returns the max round-off."""
    err = ctypes.c_double()
    _check(lib.gl_iterate_noalloc(int(p), int(N), ctypes.c_void_p(ll_in_ptr), ctypes.c_void_p(ll_out_ptr),
                                  int(iters), ctypes.byref(err), ctypes.c_void_p(stream)), "iterate_noalloc")
    return err.value


def probe_fp64_peak(device: int = 0, ms: float = 200.0) -> float:
    t = ctypes.c_double()
    _check(lib.gl_probe_fp64_peak(int(device), float(ms), ctypes.byref(t)), "probe_fp64_peak")
    return t.value


def probe_fp64_butterfly(device: int = 0, ms: float = 200.0) -> float:
    """FP64 instructions per second of the line DFTs' radix-8 butterfly (registers only)."""
    t = ctypes.c_double()
    _check(lib.gl_probe_fp64_butterfly(int(device), float(ms), ctypes.byref(t)), "probe_fp64_butterfly")
    return t.value


def describe(p: int, N: int, mode: int = MODE_FUSED, **opts) -> PlanInfo:
    """The layout a plan for (p, N) would use; needs no GPU."""
    info = PlanInfo()
    o = default_opts(mode=mode, **opts)
    _check(lib.gl_plan_describe(int(p), int(N), ctypes.byref(o), ctypes.byref(info)), f"describe p={p} N={N}")
    return info


def error_string(status: int) -> str:
    return lib.gl_error_string(int(status)).decode()


def version() -> int:
    return int(lib.gl_version())
