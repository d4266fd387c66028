"""The kernels' arithmetic helpers (gl_device.cuh), compiled for the host, against numpy.

Covers the small DFTs of every radix the line FFTs use, the integer-domain
round-half-even that replaces __double2ll_rn (gpuLucas.cu:796) with its round-off
distance, and the bit-built int -> double conversion of the weighted load
(gpuLucas.cu:757).
"""
import ctypes
import os

import numpy as np
import pytest

from gpulucas_gb300 import _build


@pytest.fixture(scope="module")
def hc():
    L = ctypes.CDLL(_build.HOSTCHECK)
    L.hc_dft.argtypes = [ctypes.c_int, ctypes.c_int, np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
    L.hc_dft.restype = ctypes.c_int
    L.hc_round.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_int)]
    L.hc_round.restype = ctypes.c_longlong
    L.hc_dbl_from_int.argtypes = [ctypes.c_int]
    L.hc_dbl_from_int.restype = ctypes.c_double
    L.hc_dice_sum.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint,
                              np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS"), ctypes.c_int, ctypes.c_int]
    L.hc_dice_sum.restype = ctypes.c_longlong
    L.hc_balanced_split.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_int)]
    return L


@pytest.mark.parametrize("R", [2, 3, 4, 5, 7, 8, 16])
@pytest.mark.parametrize("sign", [-1, 1])
def test_small_dft(hc, R, sign):
    rng = np.random.default_rng(R * 10 + sign)
    for _ in range(20):
        x = rng.standard_normal(R) + 1j * rng.standard_normal(R)
        buf = np.empty(2 * R)
        buf[0::2], buf[1::2] = x.real, x.imag
        assert hc.hc_dft(R, sign, buf) == 0
        y = buf[0::2] + 1j * buf[1::2]
        ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * R
        assert np.abs(y - ref).max() <= 1e-14 * max(1.0, np.abs(ref).max())


def _round(hc, x):
    e = ctypes.c_ulonglong()
    big = ctypes.c_int()
    r = hc.hc_round(x, ctypes.byref(e), ctypes.byref(big))
    return r, e.value / 2.0**64, big.value


def test_round_half_even_matches_rint(hc):
    rng = np.random.default_rng(7)
    vals = list(rng.standard_normal(2000) * 1e6) + list(rng.standard_normal(2000) * 2.0**45)
    vals += [0.0, -0.0, 0.5, 1.5, 2.5, -0.5, -1.5, -2.5, 3.4999999, 2.0**50 + 0.5, -(2.0**50) - 0.5,
             1e-300, -1e-300, 0.49999999999999994, 2.0**-20, 7.0, -7.0]
    for x in vals:
        r, e, big = _round(hc, x)
        assert big == 0
        assert r == int(np.rint(x)), x
        assert abs(e - abs(x - np.rint(x))) <= 2.0**-52, (x, e)


def test_round_flags_unrepresentable(hc):
    for x in [2.0**51, -(2.0**51), 2.0**60, 1e300]:
        assert _round(hc, x)[2] == 1


def test_int_to_double_exact(hc):
    for v in list(range(-70000, 70000, 7)) + [2**30, -(2**30), 2**31 - 1, -(2**31) + 1, 1, -1, 0]:
        assert hc.hc_dbl_from_int(v) == float(v)


def test_dice_matches_oracle(hc, orc):
    """llintToIrrBal<n> of the kernels vs the oracle's restatement on random products."""
    rng = np.random.default_rng(3)
    for p, N in [(44497, 2048), (100003, 5184), (12379, 640), (2976221, 163840)]:
        n = orc.slice_depth(p, N)
        LO = p // N
        bits, flags = orc.bits(p, N)
        ll = rng.integers(-(2**45), 2**45, N, dtype=np.int64)
        ll[:5] = [0, -1, 1, 2**44, -(2**44)]
        d_ref, h_ref = orc.dice(p, N, ll)
        for j in list(range(8)) + list(rng.integers(0, N, 200)) + [N - 1]:
            s = hc.hc_dice_sum(LO, n, int(flags[j]), ll, N, int(j))
            d = ctypes.c_int()
            h = ctypes.c_int()
            hc.hc_balanced_split(s, LO + int(flags[j] & 1), ctypes.byref(d), ctypes.byref(h))
            assert (d.value, h.value) == (int(d_ref[j]), int(h_ref[j])), (p, N, j)


def _level_values(R, w, sign):
    """Stored per-level twiddle values of the layered DIT: w^(R/2^l) W_(2^l)^p for
    p < max(1, 2^(l-2)), W = exp(-2 pi i/size) (conjugated for the inverse)."""
    vals = []
    l = 1
    while (1 << l) <= R:
        n_p = 1 if l == 1 else 1 << (l - 2)
        for p in range(n_p):
            vals.append(w ** (R >> l) * np.exp(-2j * np.pi * p / (1 << l)))
        l += 1
    vals = np.array(vals)
    return vals if sign < 0 else np.conj(vals)


@pytest.mark.parametrize("R", [2, 4, 8, 16])
@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("with_tw", [0, 1])
def test_layered_dit(hc, R, sign, with_tw):
    hc.hc_layered.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS"),
                              np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
    hc.hc_layered.restype = ctypes.c_int
    rng = np.random.default_rng(100 * R + 10 * with_tw + sign)
    for _ in range(20):
        x = rng.standard_normal(R) + 1j * rng.standard_normal(R)
        k, L = int(rng.integers(0, 256)), 1024
        w = np.exp(-2j * np.pi * k / L) if with_tw else 1.0
        tv = _level_values(R, w, sign)
        tbuf = np.empty(2 * len(tv))
        tbuf[0::2], tbuf[1::2] = tv.real, tv.imag
        buf = np.empty(2 * R)
        buf[0::2], buf[1::2] = x.real, x.imag
        assert hc.hc_layered(R, sign, with_tw, tbuf, buf) == 0
        y = buf[0::2] + 1j * buf[1::2]
        ww = w if sign < 0 else np.conj(w)
        xt = x * ww ** np.arange(R)
        ref = np.fft.fft(xt) if sign < 0 else np.fft.ifft(xt) * R
        assert np.abs(y - ref).max() <= 1e-14 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("radices", [[8, 8, 3, 3], [8, 8, 8, 4], [4, 3], [8, 4, 2], [3, 3, 3], [4, 4, 4, 4],
                                     [8, 8, 8, 8, 3], [16, 8, 3], [8, 5, 7], [5, 4, 3], [2, 2, 2]])
@pytest.mark.parametrize("sign", [-1, 1])
def test_line_dft_through_stage_tables(hc, radices, sign):
    """A whole line DFT through the device butterfly (stage_dft) and the product's
    stage-ordered table, in the kernels' Stockham order: twiddled radix-8/4/3 stages in
    ratio form, the others with complex values."""
    f = hc.hc_line_fft
    f.argtypes = [ctypes.c_int, np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"), ctypes.c_int,
                  ctypes.c_int, np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
    f.restype = ctypes.c_int
    L = int(np.prod(radices))
    rng = np.random.default_rng(L * 3 + sign)
    x = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    buf = np.empty(2 * L)
    buf[0::2], buf[1::2] = x.real, x.imag
    assert f(L, np.array(radices, np.int32), len(radices), sign, buf) == 0
    y = buf[0::2] + 1j * buf[1::2]
    ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * L
    assert np.abs(y - ref).max() <= 2e-15 * np.abs(ref).max()


def _ratio_twiddles(R, d):
    """w^q, q = 1..R-1, decoded from one position's stored doubles of a ratio-form stage:
    w^q = i^f rho_q (1 + i tau_q), tau stored negated where f = 1, rho from the ratios."""
    flags = int(np.array([d[{8: 3, 4: 3, 3: 3}[R]]], np.float64).view(np.int64)[0])
    if R == 8:
        tau = {2: d[0], 4: d[1], 6: d[2], 1: d[8], 5: d[9], 3: d[10], 7: d[11]}
        rho = {1: d[14], 2: d[6], 4: d[4]}
        rho[3] = d[13] * rho[1]
        rho[5] = d[7] * rho[1]
        rho[6] = d[5] * rho[2]
        rho[7] = d[12] * rho[3]
        assert d[15] == pytest.approx(rho[1] / np.sqrt(2), rel=1e-15)
    elif R == 4:
        tau = {1: d[0], 2: d[1], 3: d[2]}
        rho = {1: d[6], 2: d[4]}
        rho[3] = d[5] * rho[1]
    else:
        tau = {1: d[0], 2: d[1]}
        rho = {1: d[4], 2: d[2] * d[4]}
        assert d[5] == rho[1] / 2 and d[6] == pytest.approx(rho[1] * np.sin(2 * np.pi / 3), rel=1e-15)
    out = {}
    for q in range(1, R):
        f = (flags >> q) & 1
        t = -tau[q] if f else tau[q]
        assert abs(t) <= 1.0 and abs(rho[q]) >= np.sqrt(0.5) * (1 - 1e-15)
        out[q] = (1j ** f) * rho[q] * (1 + 1j * t)
    return out


@pytest.mark.parametrize("radices", [[8, 8, 3, 3], [8, 8, 8, 4], [4, 4, 3], [3, 8, 4]])
def test_ratio_stage_values_decode_to_twiddles(hc, radices):
    """The stored ratio-form values of every position of every twiddled radix-8/4/3 stage
    give back w^q = exp(-2 pi i k q / (Ns R)) to a few ulps, with |tau| <= 1 (the bound
    allows for the decoding's chained ratios and numpy's own rounding of the angle; a value
    in the wrong slot is off by O(1))."""
    f = hc.hc_stage_twiddles
    f.argtypes = [ctypes.c_int, np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"), ctypes.c_int,
                  ctypes.c_void_p, np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")]
    f.restype = ctypes.c_int
    L = int(np.prod(radices))
    rad = np.array(radices, np.int32)
    off = np.zeros(16, np.int32)
    n = f(L, rad, len(radices), None, off)
    tab = np.empty(2 * n)
    assert f(L, rad, len(radices), tab.ctypes.data, off) == n
    slots = {8: 8, 4: 4, 3: 4}
    Ns = 1
    for s, R in enumerate(radices):
        if Ns > 1 and R in slots:
            for k in range(Ns):
                d = np.empty(2 * slots[R])
                for v in range(slots[R]):
                    d[2 * v:2 * v + 2] = tab[2 * (off[s] + v * Ns + k):2 * (off[s] + v * Ns + k) + 2]
                w = _ratio_twiddles(R, d)
                for q, val in w.items():
                    ref = np.exp(-2j * np.pi * k * q / (Ns * R))
                    assert abs(val - ref) <= 1.5e-15, (s, R, k, q, val, ref)
        Ns *= R
