// gl_device.cuh -- device helpers shared by the Lucas-Lehmer kernels.
//
// GB300 executes FP64 add/mul/fma at about 1/70 of the FP32 rate, and the FP64
// conversions (I2F.F64, F2I.S64.F64) share that pipe.  Everything here that is not a
// butterfly therefore works on IEEE bit patterns with integer instructions:
//   * int -> double of a digit sum      (dbl_from_int)
//   * round-half-even double -> int64   (round_ll_bits), with the round-off distance
//     |x - rint(x)| as a 0.64 fixed-point integer for the max-error reduction.
// The only FP64 instructions of an iteration are the butterflies, the twiddle
// products, the pointwise square and one multiply per word for each weight.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#ifndef GL_HD
#define GL_HD __host__ __device__ __forceinline__
#endif

namespace gl {

#ifdef __CUDA_ARCH__
GL_HD int clz32(uint32_t a) { return __clz(a); }
GL_HD long long dbl_bits(double x) { return __double_as_longlong(x); }
GL_HD double bits_dbl(long long b) { return __longlong_as_double(b); }
#else
GL_HD int clz32(uint32_t a) { return a ? __builtin_clz(a) : 32; }
GL_HD long long dbl_bits(double x) {
  long long b;
  __builtin_memcpy(&b, &x, 8);
  return b;
}
GL_HD double bits_dbl(long long b) {
  double x;
  __builtin_memcpy(&x, &b, 8);
  return x;
}
#endif

struct __align__(16) cplx {
  double re, im;
};

GL_HD cplx mk(double r, double i) { cplx c; c.re = r; c.im = i; return c; }
GL_HD cplx add(cplx a, cplx b) { return mk(a.re + b.re, a.im + b.im); }
GL_HD cplx sub(cplx a, cplx b) { return mk(a.re - b.re, a.im - b.im); }
// a * b, 2 DMUL + 2 DFMA
GL_HD cplx cmul(cplx a, cplx b) {
  return mk(fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re));
}
// a * conj(b)
GL_HD cplx cmulc(cplx a, cplx b) {
  return mk(fma(a.re, b.re, a.im * b.im), fma(a.im, b.re, -a.re * b.im));
}
// multiply by S*i (S = -1: -i, S = +1: +i): a swap and a sign, no FP64 arithmetic
template <int S>
GL_HD cplx mul_si(cplx a) {
  return S < 0 ? mk(a.im, -a.re) : mk(-a.im, a.re);
}
GL_HD cplx conj(cplx a) { return mk(a.re, -a.im); }

// ---------------------------------------------------------------------------
// small DFTs, y_k = sum_n x_n w^(nk), w = exp(S 2 pi i / R); S = -1 forward
// ---------------------------------------------------------------------------
template <int S>
GL_HD void dft2(cplx* x) {
  cplx a = x[0], b = x[1];
  x[0] = add(a, b);
  x[1] = sub(a, b);
}

template <int S>
GL_HD void dft4(cplx* x) {
  cplx s02 = add(x[0], x[2]), d02 = sub(x[0], x[2]);
  cplx s13 = add(x[1], x[3]), d13 = mul_si<S>(sub(x[1], x[3]));
  x[0] = add(s02, s13);
  x[2] = sub(s02, s13);
  x[1] = add(d02, d13);
  x[3] = sub(d02, d13);
}

#define GL_SQRT1_2 0.70710678118654752440
#define GL_C8 0.92387953251128675613   // cos(pi/8)
#define GL_S8 0.38268343236508977173   // sin(pi/8)
#define GL_C3 0.86602540378443864676   // sin(2pi/3)

template <int S>
GL_HD void dft8(cplx* x) {
  // even/odd split into two DFT4, then w8^k on the odd half
  cplx e[4] = {x[0], x[2], x[4], x[6]};
  cplx o[4] = {x[1], x[3], x[5], x[7]};
  dft4<S>(e);
  dft4<S>(o);
  // w8^1 = (1 + S i)/sqrt2, w8^2 = S i, w8^3 = (-1 + S i)/sqrt2
  cplx o1 = mk((o[1].re - S * o[1].im) * GL_SQRT1_2, (o[1].im + S * o[1].re) * GL_SQRT1_2);
  cplx o2 = mul_si<S>(o[2]);
  cplx o3 = mk((-o[3].re - S * o[3].im) * GL_SQRT1_2, (-o[3].im + S * o[3].re) * GL_SQRT1_2);
  x[0] = add(e[0], o[0]);
  x[4] = sub(e[0], o[0]);
  x[1] = add(e[1], o1);
  x[5] = sub(e[1], o1);
  x[2] = add(e[2], o2);
  x[6] = sub(e[2], o2);
  x[3] = add(e[3], o3);
  x[7] = sub(e[3], o3);
}

// w16^e for e in {1, 3} (the others reduce to w8 / S i)
template <int S>
GL_HD cplx mul_w16_1(cplx a) {  // (C8 + S i S8)
  return mk(fma(a.re, GL_C8, -S * a.im * GL_S8), fma(a.im, GL_C8, S * a.re * GL_S8));
}
template <int S>
GL_HD cplx mul_w16_3(cplx a) {  // (S8 + S i C8)
  return mk(fma(a.re, GL_S8, -S * a.im * GL_C8), fma(a.im, GL_S8, S * a.re * GL_C8));
}
template <int S>
GL_HD cplx mul_w8_1(cplx a) {
  return mk((a.re - S * a.im) * GL_SQRT1_2, (a.im + S * a.re) * GL_SQRT1_2);
}
template <int S>
GL_HD cplx mul_w8_3(cplx a) {
  return mk((-a.re - S * a.im) * GL_SQRT1_2, (-a.im + S * a.re) * GL_SQRT1_2);
}

template <int S>
GL_HD void dft16(cplx* x) {
  // n = 4 n1 + n2, k = k1 + 4 k2
  cplx a[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    cplx t[4] = {x[n2], x[4 + n2], x[8 + n2], x[12 + n2]};
    dft4<S>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[n2][k1] = t[k1];
  }
  // twiddles w16^(n2 k1)
  a[1][1] = mul_w16_1<S>(a[1][1]);
  a[1][2] = mul_w8_1<S>(a[1][2]);
  a[1][3] = mul_w16_3<S>(a[1][3]);
  a[2][1] = mul_w8_1<S>(a[2][1]);
  a[2][2] = mul_si<S>(a[2][2]);
  a[2][3] = mul_w8_3<S>(a[2][3]);
  a[3][1] = mul_w16_3<S>(a[3][1]);
  a[3][2] = mul_w8_3<S>(a[3][2]);
  // w16^9 = -w16^1
  {
    cplx t = mul_w16_1<S>(a[3][3]);
    a[3][3] = mk(-t.re, -t.im);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cplx t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
    dft4<S>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) x[k1 + 4 * k2] = t[k2];
  }
}

template <int S>
GL_HD void dft3(cplx* x) {
  cplx t1 = add(x[1], x[2]);
  cplx d = sub(x[1], x[2]);
  cplx t2 = mk(fma(-0.5, t1.re, x[0].re), fma(-0.5, t1.im, x[0].im));
  // i * S*sin(2pi/3) * d
  cplx t3 = mk(-S * GL_C3 * d.im, S * GL_C3 * d.re);
  x[0] = add(x[0], t1);
  x[1] = add(t2, t3);
  x[2] = sub(t2, t3);
}

#define GL_C51 0.30901699437494742410   // cos(2pi/5)
#define GL_C52 -0.80901699437494742410  // cos(4pi/5)
#define GL_S51 0.95105651629515357212   // sin(2pi/5)
#define GL_S52 0.58778525229247312917   // sin(4pi/5)

template <int S>
GL_HD void dft5(cplx* x) {
  cplx t1 = add(x[1], x[4]), t2 = add(x[2], x[3]);
  cplx t3 = sub(x[1], x[4]), t4 = sub(x[2], x[3]);
  cplx x0 = x[0];
  cplx a1 = mk(fma(GL_C52, t2.re, fma(GL_C51, t1.re, x0.re)), fma(GL_C52, t2.im, fma(GL_C51, t1.im, x0.im)));
  cplx a2 = mk(fma(GL_C51, t2.re, fma(GL_C52, t1.re, x0.re)), fma(GL_C51, t2.im, fma(GL_C52, t1.im, x0.im)));
  // b1 = S(s1 t3 + s2 t4), b2 = S(s2 t3 - s1 t4); y1 = a1 + i b1
  cplx b1 = mk(S * fma(GL_S51, t3.re, GL_S52 * t4.re), S * fma(GL_S51, t3.im, GL_S52 * t4.im));
  cplx b2 = mk(S * fma(GL_S52, t3.re, -GL_S51 * t4.re), S * fma(GL_S52, t3.im, -GL_S51 * t4.im));
  x[0] = add(x0, add(t1, t2));
  x[1] = mk(a1.re - b1.im, a1.im + b1.re);
  x[4] = mk(a1.re + b1.im, a1.im - b1.re);
  x[2] = mk(a2.re - b2.im, a2.im + b2.re);
  x[3] = mk(a2.re + b2.im, a2.im - b2.re);
}

#define GL_C71 0.62348980185873353053   // cos(2pi/7)
#define GL_C72 -0.22252093395631440429  // cos(4pi/7)
#define GL_C73 -0.90096886790241912624  // cos(6pi/7)
#define GL_S71 0.78183148246802980871
#define GL_S72 0.97492791218182360702
#define GL_S73 0.43388373911755812048

template <int S>
GL_HD void dft7(cplx* x) {
  cplx x0 = x[0];
  cplx p1 = add(x[1], x[6]), m1 = sub(x[1], x[6]);
  cplx p2 = add(x[2], x[5]), m2 = sub(x[2], x[5]);
  cplx p3 = add(x[3], x[4]), m3 = sub(x[3], x[4]);
  // a_k = x0 + sum_j cos(2 pi jk/7) p_j ; b_k = S sum_j sin(2 pi jk/7) m_j
  cplx a1 = mk(x0.re + GL_C71 * p1.re + GL_C72 * p2.re + GL_C73 * p3.re,
               x0.im + GL_C71 * p1.im + GL_C72 * p2.im + GL_C73 * p3.im);
  cplx a2 = mk(x0.re + GL_C72 * p1.re + GL_C73 * p2.re + GL_C71 * p3.re,
               x0.im + GL_C72 * p1.im + GL_C73 * p2.im + GL_C71 * p3.im);
  cplx a3 = mk(x0.re + GL_C73 * p1.re + GL_C71 * p2.re + GL_C72 * p3.re,
               x0.im + GL_C73 * p1.im + GL_C71 * p2.im + GL_C72 * p3.im);
  cplx b1 = mk(S * (GL_S71 * m1.re + GL_S72 * m2.re + GL_S73 * m3.re),
               S * (GL_S71 * m1.im + GL_S72 * m2.im + GL_S73 * m3.im));
  cplx b2 = mk(S * (GL_S72 * m1.re - GL_S73 * m2.re - GL_S71 * m3.re),
               S * (GL_S72 * m1.im - GL_S73 * m2.im - GL_S71 * m3.im));
  cplx b3 = mk(S * (GL_S73 * m1.re - GL_S71 * m2.re + GL_S72 * m3.re),
               S * (GL_S73 * m1.im - GL_S71 * m2.im + GL_S72 * m3.im));
  x[0] = add(x0, add(p1, add(p2, p3)));
  x[1] = mk(a1.re - b1.im, a1.im + b1.re);
  x[6] = mk(a1.re + b1.im, a1.im - b1.re);
  x[2] = mk(a2.re - b2.im, a2.im + b2.re);
  x[5] = mk(a2.re + b2.im, a2.im - b2.re);
  x[3] = mk(a3.re - b3.im, a3.im + b3.re);
  x[4] = mk(a3.re + b3.im, a3.im - b3.re);
}

// ---------------------------------------------------------------------------
// Layered radix-2 DIT of R = 2^r points with an external twiddle (Linzer-Feig
// style FMA merging).  y_p = sum_q x_q (w W_R^p)^q with W_R = exp(S 2 pi i/R):
// after the bit-reversed input order, level l (sub-DFT size 2^l) combines
// (a, c) -> (a + t c, a - t c) with t = w^(R/2^l) W_(2^l)^p.  For p in the upper
// quarter t is S i times the value for p - 2^(l-2), so a level stores only
// max(1, 2^(l-2)) values.  a + t c costs 4 FMA and a - t c = 2a - (a + t c) 2 more;
// with t = 1 or S i a butterfly is 4 adds.
// ---------------------------------------------------------------------------
// (a, c) -> (a + c, a - c)
GL_HD void bf_one(cplx& a, cplx& c) {
  const cplx u = add(a, c);
  c = sub(a, c);
  a = u;
}
// (a, c) -> (a + S i c, a - S i c)
template <int S>
GL_HD void bf_si(cplx& a, cplx& c) {
  const cplx sc = mul_si<S>(c);
  const cplx u = add(a, sc);
  c = sub(a, sc);
  a = u;
}
// (a, c) -> (a + t c, a - t c)
GL_HD void bf_tw(cplx& a, cplx& c, const cplx t) {
  const double ur = fma(t.re, c.re, fma(-t.im, c.im, a.re));
  const double ui = fma(t.re, c.im, fma(t.im, c.re, a.im));
  c = mk(fma(2.0, a.re, -ur), fma(2.0, a.im, -ui));
  a = mk(ur, ui);
}
// (a, c) -> (a + S i t c, a - S i t c)
template <int S>
GL_HD void bf_si_tw(cplx& a, cplx& c, const cplx t) {
  // S i t c = S i (tr cr - ti ci) - S (tr ci + ti cr)
  const double ur = fma(-S * t.re, c.im, fma(-S * t.im, c.re, a.re));
  const double ui = fma(S * t.re, c.re, fma(-S * t.im, c.im, a.im));
  c = mk(fma(2.0, a.re, -ur), fma(2.0, a.im, -ui));
  a = mk(ur, ui);
}

__host__ __device__ constexpr int ilog2c(int r) { return r <= 1 ? 0 : 1 + ilog2c(r >> 1); }
// reverse the low `bits` (<= 4) bits of i; plain arithmetic, so an unrolled loop index
// folds it to a constant and the register arrays stay statically indexed
GL_HD int bitrev4(int i, int bits) {
  const int x = ((i & 1) << 3) | ((i & 2) << 1) | ((i & 4) >> 1) | ((i & 8) >> 3);
  return x >> (4 - bits);
}

// exp(S 2 pi i p / size) for the constant (first-stage) twiddles, size in {8, 16}
template <int S>
GL_HD cplx wconst(int p, int size) {
  // only called with p < size/4 (the S i symmetry covers the rest)
  if (size == 8) return mk(GL_SQRT1_2, S * GL_SQRT1_2);  // p == 1
  // size 16: p = 1, 2, 3
  if (p == 1) return mk(GL_C8, S * GL_S8);
  if (p == 2) return mk(GL_SQRT1_2, S * GL_SQRT1_2);
  return mk(GL_S8, S * GL_C8);
}

// One level (sub-DFT size 2^LV) of the layered DIT; every trip count is a
// compile-time constant so the register arrays stay statically indexed.
template <int R, int S, bool TW, int LV>
GL_HD void dit_level(cplx* y, const cplx* tv) {
  constexpr int half = 1 << (LV - 1);
  constexpr int quarter = half >> 1;
  constexpr int vbase = LV == 1 ? 0 : (1 << (LV - 2));
#pragma unroll
  for (int b = 0; b < R; b += 2 * half) {
#pragma unroll
    for (int p = 0; p < half; ++p) {
      const bool si = LV >= 2 && p >= quarter;
      const int pp = si ? p - quarter : p;
      if (TW) {
        const cplx t = tv[vbase + pp];
        if (si) bf_si_tw<S>(y[b + p], y[b + p + half], t);
        else bf_tw(y[b + p], y[b + p + half], t);
      } else if (pp == 0) {
        if (si) bf_si<S>(y[b + p], y[b + p + half]);
        else bf_one(y[b + p], y[b + p + half]);
      } else {
        const cplx t = wconst<S>(pp, 2 * half);
        if (si) bf_si_tw<S>(y[b + p], y[b + p + half], t);
        else bf_tw(y[b + p], y[b + p + half], t);
      }
    }
  }
}

// TW = false: no external twiddle (constant W factors only).  TW = true: tv holds the
// stage's stored values (already conjugated for S = +1).
template <int R, int S, bool TW>
GL_HD void layered_dit(cplx* x, const cplx* tv) {
  constexpr int r = ilog2c(R);
  cplx y[R];
#pragma unroll
  for (int i = 0; i < R; ++i) y[i] = x[bitrev4(i, r)];
  dit_level<R, S, TW, 1>(y, tv);
  if constexpr (R >= 4) dit_level<R, S, TW, 2>(y, tv);
  if constexpr (R >= 8) dit_level<R, S, TW, 3>(y, tv);
  if constexpr (R >= 16) dit_level<R, S, TW, 4>(y, tv);
#pragma unroll
  for (int i = 0; i < R; ++i) x[i] = y[i];
}

template <int R, int S>
GL_HD void dft(cplx* x) {
  if constexpr (R == 2) dft2<S>(x);
  else if constexpr (R == 3) dft3<S>(x);
  else if constexpr (R == 4) dft4<S>(x);
  else if constexpr (R == 5) dft5<S>(x);
  else if constexpr (R == 7) dft7<S>(x);
  else if constexpr (R == 8) dft8<S>(x);
  else if constexpr (R == 16) dft16<S>(x);
}

// ---------------------------------------------------------------------------
// Twiddled radix-8, -4 and -3 stages in ratio form, after S. Goedecker, "Fast radix 2,
// 3, 4, and 5 kernels for fast Fourier transformations on computers with overlapping
// multiply-add instructions", SIAM J. Sci. Comput. 18 (1997) 1605-1611.  Each external
// twiddle w^q (forward direction) is stored as
//     w^q = i^f rho_q (1 + i tau_q),   |tau_q| <= 1, f in {0, 1}, |rho_q| >= 1/sqrt2:
// the input is rotated by i^f (register selects and a sign bit, no FP64 instruction),
// multiplied by (1 + i tau_q) (2 FMA), and the real factors rho_q ride in the FMAs of
// the DFT that follows as ratios of the two inputs each sum combines (sigma = rho_a /
// rho_b), so every sum or difference costs 2 FMA.  FP64 instructions per butterfly:
// radix 8: 66 (layered DIT with complex twiddles: 72), radix 4: 22 (24), radix 3: 16
// (two complex products and DFT_3: 22).  The inverse direction (S = +1) uses the same
// stored values for conj(w^q): rotation by -i, tau -> -tau.
//
// Stored doubles per butterfly position (pairs of them per 16-byte slot), tau_q stored
// with the sign of f folded in (-tau_q where f = 1):
//   R = 8: tau2, tau4, tau6, flags, rho4, rho6/rho2, rho2, rho5/rho1, tau1, tau5, tau3,
//          tau7, rho7/rho3, rho3/rho1, rho1, rho1/sqrt2
//   R = 4: tau1, tau2, tau3, flags, rho2, rho3/rho1, rho1, 0
//   R = 3: tau1, tau2, rho2/rho1, flags, rho1, rho1/2, rho1 sin(2pi/3), 0
// flags: bit q = f of w^q, held as the bit pattern of the double.
// ---------------------------------------------------------------------------
// Sign of x flipped when f == 1, by an integer instruction on the high word.  Inline PTX
// keeps the compiler from turning a sign-bit XOR back into an FP64 negation, which it
// would issue as a DADD when the negated value feeds a select.
GL_HD double flip_sign_if(double x, unsigned f) {
#ifdef __CUDA_ARCH__
  int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  asm("xor.b32 %0, %0, %1;" : "+r"(hi) : "r"(f << 31));
  return __hiloint2double(hi, lo);
#else
  return bits_dbl(dbl_bits(x) ^ (long long)((unsigned long long)f << 63));
#endif
}

// Forward (S = -1): (1 + i tau) i^f x; inverse (S = +1): (1 - i tau) (-i)^f x.  The table
// holds t = tau for f = 0 and t = -tau for f = 1; with (a, b) = (re, im) or (im, re):
//   forward  u = (+-(a - t b), b + t a),   inverse  u = (a + t b, +-(b - t a)),
// the sign flipped for f = 1.  2 FMA and integer instructions (selects, one XOR).
template <int S>
GL_HD cplx prerot(cplx x, double t, unsigned f) {
  const double a = f ? x.im : x.re, b = f ? x.re : x.im;
  if (S < 0) return mk(flip_sign_if(fma(-t, b, a), f), fma(t, a, b));
  return mk(fma(t, b, a), flip_sign_if(fma(-t, a, b), f));
}
// a + l b, l real: 2 FMA
GL_HD cplx axpy(double l, cplx b, cplx a) { return mk(fma(l, b.re, a.re), fma(l, b.im, a.im)); }
// a + S i l b, l real: 2 FMA
template <int S>
GL_HD cplx axpy_si(double l, cplx b, cplx a) {
  return mk(fma(S < 0 ? l : -l, b.im, a.re), fma(S < 0 ? -l : l, b.re, a.im));
}
GL_HD unsigned flag_bits(double v) { return (unsigned)dbl_bits(v); }

// slot(i) returns the i-th 16-byte slot of this butterfly's stored values; the values
// are read where they are used, so few of them are live at once.  Radix 8 runs the even
// inputs' DFT_4, then the odd inputs', then the combining level, so at most the even
// results and the odd inputs are live between the halves.
template <int S, typename Slot>
GL_HD void ratio_r8(cplx* v, const Slot& slot) {
  const cplx s1 = slot(1);
  const unsigned fl = flag_bits(s1.im);
  // even inputs: DFT_4 of (v0, rho2 u2, rho4 u4, rho6 u6)
  cplx e0, e1, e2, e3;
  double sig5;
  {
    const cplx s0 = slot(0), s2 = slot(2), s3 = slot(3);
    sig5 = s3.im;
    const cplx u4 = prerot<S>(v[4], s0.im, (fl >> 4) & 1);
    const cplx a0 = axpy(s2.re, u4, v[0]), a1 = axpy(-s2.re, u4, v[0]);
    const cplx u2 = prerot<S>(v[2], s0.re, (fl >> 2) & 1);
    const cplx u6 = prerot<S>(v[6], s1.re, (fl >> 6) & 1);
    const cplx b0 = axpy(s2.im, u6, u2), b1 = axpy(-s2.im, u6, u2);
    e0 = axpy(s3.re, b0, a0);
    e2 = axpy(-s3.re, b0, a0);
    e1 = axpy_si<S>(s3.re, b1, a1);
    e3 = axpy_si<S>(-s3.re, b1, a1);
  }
  // odd inputs over rho1: DFT_4 of (u1, (rho3/rho1) u3, (rho5/rho1) u5, (rho7/rho1) u7)
  cplx o0, o1, o2, o3;
  {
    const cplx s4 = slot(4), s5 = slot(5), s6 = slot(6);
    const cplx u1 = prerot<S>(v[1], s4.re, (fl >> 1) & 1);
    const cplx u5 = prerot<S>(v[5], s4.im, (fl >> 5) & 1);
    const cplx c0 = axpy(sig5, u5, u1), c1 = axpy(-sig5, u5, u1);
    const cplx u3 = prerot<S>(v[3], s5.re, (fl >> 3) & 1);
    const cplx u7 = prerot<S>(v[7], s5.im, (fl >> 7) & 1);
    const cplx d0 = axpy(s6.re, u7, u3), d1 = axpy(-s6.re, u7, u3);
    o0 = axpy(s6.im, d0, c0);
    o2 = axpy(-s6.im, d0, c0);
    o1 = axpy_si<S>(s6.im, d1, c1);
    o3 = axpy_si<S>(-s6.im, d1, c1);
  }
  // y_p = E_p + W8^p rho1 O_p, y_(p+4) = E_p - W8^p rho1 O_p
  const cplx s7 = slot(7);
  v[0] = axpy(s7.re, o0, e0);
  v[4] = axpy(-s7.re, o0, e0);
  v[2] = axpy_si<S>(s7.re, o2, e2);
  v[6] = axpy_si<S>(-s7.re, o2, e2);
  // W8 = (1 + S i)/sqrt2, W8^3 = (-1 + S i)/sqrt2; s7.im = rho1/sqrt2
  const cplx t1 = S < 0 ? mk(o1.re + o1.im, o1.im - o1.re) : mk(o1.re - o1.im, o1.im + o1.re);
  const cplx t3 = S < 0 ? mk(o3.im - o3.re, -o3.im - o3.re) : mk(-o3.re - o3.im, o3.re - o3.im);
  v[1] = axpy(s7.im, t1, e1);
  v[5] = axpy(-s7.im, t1, e1);
  v[3] = axpy(s7.im, t3, e3);
  v[7] = axpy(-s7.im, t3, e3);
}

template <int S, typename Slot>
GL_HD void ratio_r4(cplx* v, const Slot& slot) {
  const cplx s0 = slot(0), s1 = slot(1);
  const unsigned fl = flag_bits(s1.im);
  const cplx u1 = prerot<S>(v[1], s0.re, (fl >> 1) & 1);
  const cplx u2 = prerot<S>(v[2], s0.im, (fl >> 2) & 1);
  const cplx u3 = prerot<S>(v[3], s1.re, (fl >> 3) & 1);
  const cplx s2 = slot(2), s3 = slot(3);
  const cplx a0 = axpy(s2.re, u2, v[0]), a1 = axpy(-s2.re, u2, v[0]);
  const cplx b0 = axpy(s2.im, u3, u1), b1 = axpy(-s2.im, u3, u1);
  v[0] = axpy(s3.re, b0, a0);
  v[2] = axpy(-s3.re, b0, a0);
  v[1] = axpy_si<S>(s3.re, b1, a1);
  v[3] = axpy_si<S>(-s3.re, b1, a1);
}

template <int S, typename Slot>
GL_HD void ratio_r3(cplx* v, const Slot& slot) {
  const cplx s0 = slot(0), s1 = slot(1);
  const unsigned fl = flag_bits(s1.im);
  const cplx u1 = prerot<S>(v[1], s0.re, (fl >> 1) & 1);
  const cplx u2 = prerot<S>(v[2], s0.im, (fl >> 2) & 1);
  const cplx s2 = slot(2), s3 = slot(3);
  const cplx t = axpy(s1.re, u2, u1), d = axpy(-s1.re, u2, u1);
  const cplx m = axpy(-s2.im, t, v[0]);
  v[0] = axpy(s2.re, t, v[0]);
  v[1] = axpy_si<S>(s3.re, d, m);
  v[2] = axpy_si<S>(-s3.re, d, m);
}

// Stored 16-byte slots per butterfly position of a twiddled stage of radix R.
template <int R>
GL_HD constexpr int stage_slots() {
  return R == 8 ? 8 : (R == 4 || R == 3) ? 4 : ((R & (R - 1)) == 0 ? (R == 2 ? 1 : R / 2) : R - 1);
}

// One butterfly of a Stockham stage: DFT_R of v[q] w^q (w^q = 1 in the first stage,
// Ns == 1).  slot(i) reads the stage's i-th stored slot of this butterfly position.
// Radices 8, 4, 3 use the ratio form; 2 and 16 the layered DIT with complex values
// (level values w^(R/2^l) W_(2^l)^p, conjugated here for S = +1); 5 and 7 a complex
// product per input and DFT_R.
template <int R, int S, typename Slot>
GL_HD void stage_dft(cplx* v, bool twiddled, const Slot& slot) {
  constexpr bool POW2 = (R & (R - 1)) == 0;
  if (!twiddled) {
    if constexpr (POW2) layered_dit<R, S, false>(v, nullptr);
    else dft<R, S>(v);
  } else if constexpr (R == 8) {
    ratio_r8<S>(v, slot);
  } else if constexpr (R == 4) {
    ratio_r4<S>(v, slot);
  } else if constexpr (R == 3) {
    ratio_r3<S>(v, slot);
  } else {
    constexpr int NV = stage_slots<R>();
    cplx tv[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const cplx t = slot(i);
      tv[i] = S < 0 ? t : conj(t);
    }
    if constexpr (POW2) {
      layered_dit<R, S, true>(v, tv);
    } else {
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tv[q - 1]);
      dft<R, S>(v);
    }
  }
}

// ---------------------------------------------------------------------------
// integer-domain conversions
// ---------------------------------------------------------------------------

// exact double of a 32-bit integer, built from its bits (no I2F.F64)
GL_HD double dbl_from_int(int v) {
  if (v == 0) return 0.0;
  uint32_t a = v < 0 ? (uint32_t)(-v) : (uint32_t)v;
  int top = 31 - clz32(a);                               // position of the leading 1
  uint64_t mant = ((uint64_t)a << (52 - top)) & 0x000FFFFFFFFFFFFFull;
  uint64_t bits = ((uint64_t)(v < 0) << 63) | ((uint64_t)(top + 1023) << 52) | mant;
  return bits_dbl((long long)bits);
}

// Round x half-to-even to int64 (as __double2ll_rn) using integer instructions.
// *err64 receives |x - rint(x)| * 2^64 (so 0.5 -> 2^63), and *big is set when
// |x| >= 2^51, past which the products can no longer be trusted.
GL_HD long long round_ll_bits(double x, unsigned long long* err64, int* big) {
  uint64_t b = (uint64_t)dbl_bits(x);
  int e = (int)((b >> 52) & 0x7FF);
  uint64_t mant = (b & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(e != 0) << 52);
  int E = e - 1023;  // x = mant * 2^(E-52)
  bool neg = (b >> 63) != 0;
  long long r;
  unsigned long long er;
  if (E >= 51) {
    *big = 1;
    r = 0;
    er = 0;
  } else if (E < -1) {
    // |x| < 0.5: rounds to 0, distance |x| = mant * 2^(E-52); scaled by 2^64: mant * 2^(E+12)
    r = 0;
    int s = E + 12;
    er = (e == 0) ? 0ull : (s >= 0 ? (unsigned long long)(mant << s) : (unsigned long long)(s > -64 ? mant >> (-s) : 0));
  } else {
    int sh = 52 - E;  // 2..53 fractional bits
    uint64_t ip = mant >> sh;
    uint64_t rem = mant & ((1ull << sh) - 1);
    uint64_t half = 1ull << (sh - 1);
    uint64_t dist = rem;
    if (rem > half || (rem == half && (ip & 1))) {
      ip += 1;
      dist = (1ull << sh) - rem;
    }
    r = neg ? -(long long)ip : (long long)ip;
    er = (unsigned long long)(dist << (64 - sh));
  }
  *err64 = er;
  return r;
}

// ---------------------------------------------------------------------------
// Dicing: llintToIrrBal<n> (IrrBaseBalanced.cu:52-110) for one word.
// ll_at(i) returns the product of word j - i (i = 0..n), f is bitsPerWord8[j].
// Returns the digit sum before the balanced split.
// ---------------------------------------------------------------------------
template <typename F>
GL_HD long long dice_sum(int LO, int n, uint32_t f, F ll_at) {
  int isHi = f & 1;
  long long mask = (1ll << (LO + isHi)) - 1;
  long long v = ll_at(0);
  long long sum = v < 0 ? -((-v) & mask) : (v & mask);
  int shift = 0;
  for (int i = 1; i <= n; ++i) {
    shift += LO + ((f >> i) & 1);
    if (shift >= 63) break;  // nothing of a 63-bit magnitude lies this high
    long long w = ll_at(i);
    long long s = w < 0 ? -(((-w) >> shift) & mask) : ((w >> shift) & mask);
    sum += s;
  }
  return sum;
}

// balanced split of a digit sum: hi = carry (int8), digit = sum - hi * base
GL_HD void balanced_split(long long sum, int bits, int* digit, int* hi) {
  long long half = 1ll << (bits - 1);
  long long h = 0;
  if (sum < -half) h = -((-sum + half) >> bits);
  else if (sum >= half) h = (sum + half) >> bits;
  *digit = (int)(sum - h * (1ll << bits));
  *hi = (int)h;
}

}  // namespace gl
