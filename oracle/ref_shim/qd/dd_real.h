/*
 * qd/dd_real.h -- a stand-in for the QD library's double-double header, written for this
 * project so that the reference gpuLucas program can be compiled and run as an oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library includes this file.  The
 * reference includes <qd/dd_real.h> (gpuLucas.cu:153) for one routine,
 * computeWeightVectors (gpuLucas.cu:673-686), which needs: dd_real(int), dd_real(double),
 * dd * dd, dd / dd, dd - dd, double / dd, ceil(dd), pow(dd, dd) and to_double(dd).  QD
 * (2.3.x) is not installed on either machine, so this header provides those operations
 * with the published double-double algorithms:
 *
 *   - error-free sum and product: Knuth's TwoSum (TAOCP vol. 2, 4.2.2), Dekker's
 *     Fast2Sum (Numer. Math. 18, 1971), the product error term by one fused multiply-add;
 *   - division: long division with three quotient digits, each refined against the
 *     exact remainder;
 *   - exp: x = k ln2 + r, |r| <= ln2/2, r scaled by 2^-10, Taylor series of e^s - 1, then
 *     ten squarings of (1 + t) kept as t' = 2t + t^2 so the small part keeps its bits;
 *   - log: one Newton step x + a e^-x - 1 from the double logarithm;
 *   - pow(a, b) = exp(b log a) (pow(2, b) uses the ln 2 constant directly).
 *
 * Every result is accurate to a few units of 2^-104 relative; rounded to double it is
 * the correctly rounded value except within that distance of a rounding tie.  The CPU
 * suite checks the weights this header produces against mpmath at 140 bits.
 *
 * Build the reference with -ffp-contract=off for the host code so the error-free
 * transformations are not contracted into different fused operations.
 */
#ifndef GL_REF_SHIM_DD_REAL_H
#define GL_REF_SHIM_DD_REAL_H

#include <cmath>

class dd_real {
 public:
  double x[2];

  dd_real() { x[0] = 0.0; x[1] = 0.0; }
  dd_real(double hi) { x[0] = hi; x[1] = 0.0; }
  dd_real(int v) { x[0] = static_cast<double>(v); x[1] = 0.0; }
  dd_real(double hi, double lo) { x[0] = hi; x[1] = lo; }
};

namespace dd_shim {

/* s + e == a + b exactly, given |a| >= |b|. */
inline dd_real fast_two_sum(double a, double b) {
  double s = a + b;
  double e = b - (s - a);
  return dd_real(s, e);
}

/* s + e == a + b exactly, any order. */
inline dd_real two_sum(double a, double b) {
  double s = a + b;
  double bv = s - a;
  double av = s - bv;
  return dd_real(s, (a - av) + (b - bv));
}

/* p + e == a * b exactly. */
inline dd_real two_prod(double a, double b) {
  double p = a * b;
  return dd_real(p, std::fma(a, b, -p));
}

inline dd_real add(const dd_real& a, const dd_real& b) {
  dd_real s = two_sum(a.x[0], b.x[0]);
  dd_real t = two_sum(a.x[1], b.x[1]);
  double lo = s.x[1] + t.x[0];
  s = fast_two_sum(s.x[0], lo);
  lo = s.x[1] + t.x[1];
  return fast_two_sum(s.x[0], lo);
}

inline dd_real neg(const dd_real& a) { return dd_real(-a.x[0], -a.x[1]); }

inline dd_real mul(const dd_real& a, const dd_real& b) {
  dd_real p = two_prod(a.x[0], b.x[0]);
  double lo = p.x[1] + (a.x[0] * b.x[1] + a.x[1] * b.x[0]);
  return fast_two_sum(p.x[0], lo);
}

inline dd_real mul_d(const dd_real& a, double b) {
  dd_real p = two_prod(a.x[0], b);
  double lo = p.x[1] + a.x[1] * b;
  return fast_two_sum(p.x[0], lo);
}

inline dd_real div(const dd_real& a, const dd_real& b) {
  double q1 = a.x[0] / b.x[0];
  dd_real r = add(a, neg(mul_d(b, q1)));
  double q2 = r.x[0] / b.x[0];
  r = add(r, neg(mul_d(b, q2)));
  double q3 = r.x[0] / b.x[0];
  dd_real q = fast_two_sum(q1, q2);
  return add(q, dd_real(q3));
}

inline dd_real ldexp2(const dd_real& a, int e) { return dd_real(std::ldexp(a.x[0], e), std::ldexp(a.x[1], e)); }

/* ln 2 = 0.693147180559945309417232121458176568..., split into two doubles. */
inline dd_real ln2() { return dd_real(0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56); }

inline dd_real exp(const dd_real& a) {
  if (a.x[0] > 709.0) return dd_real(HUGE_VAL);
  if (a.x[0] < -745.0) return dd_real(0.0);
  if (a.x[0] == 0.0 && a.x[1] == 0.0) return dd_real(1.0);
  double k = std::nearbyint(a.x[0] / ln2().x[0]);
  dd_real r = add(a, neg(mul_d(ln2(), k)));  /* |r| <= ln2/2 (plus rounding) */
  dd_real s = ldexp2(r, -10);                /* |s| < 3.4e-4 */
  /* t = e^s - 1 = s + s^2/2! + ... ; terms fall below 2^-110 relative after ~12 */
  dd_real term = s, t = s;
  for (int n = 2; n <= 14; ++n) {
    term = div(mul(term, s), dd_real(static_cast<double>(n)));
    t = add(t, term);
    if (std::fabs(term.x[0]) < 1e-36) break;
  }
  /* (1 + t)^(2^10) - 1, each squaring as 2t + t^2 */
  for (int i = 0; i < 10; ++i) t = add(ldexp2(t, 1), mul(t, t));
  return ldexp2(add(dd_real(1.0), t), static_cast<int>(k));
}

inline dd_real log(const dd_real& a) {
  if (a.x[0] <= 0.0) return dd_real(std::nan(""));
  double x0 = std::log(a.x[0]);
  /* x1 = x0 + a e^-x0 - 1: one Newton step doubles the correct bits */
  dd_real e = exp(dd_real(-x0));
  return add(dd_real(x0), add(mul(a, e), dd_real(-1.0)));
}

}  // namespace dd_shim

inline dd_real operator+(const dd_real& a, const dd_real& b) { return dd_shim::add(a, b); }
inline dd_real operator-(const dd_real& a, const dd_real& b) { return dd_shim::add(a, dd_shim::neg(b)); }
inline dd_real operator-(const dd_real& a) { return dd_shim::neg(a); }
inline dd_real operator*(const dd_real& a, const dd_real& b) { return dd_shim::mul(a, b); }
inline dd_real operator/(const dd_real& a, const dd_real& b) { return dd_shim::div(a, b); }
inline dd_real operator/(double a, const dd_real& b) { return dd_shim::div(dd_real(a), b); }
inline dd_real operator/(const dd_real& a, double b) { return dd_shim::div(a, dd_real(b)); }
inline dd_real operator*(double a, const dd_real& b) { return dd_shim::mul_d(b, a); }
inline dd_real operator*(const dd_real& a, double b) { return dd_shim::mul_d(a, b); }

inline dd_real ceil(const dd_real& a) {
  double hi = std::ceil(a.x[0]);
  double lo = 0.0;
  if (hi == a.x[0]) {
    /* the high part is an integer: the low part decides */
    lo = std::ceil(a.x[1]);
    return dd_shim::fast_two_sum(hi, lo);
  }
  return dd_real(hi, lo);
}

inline dd_real floor(const dd_real& a) {
  double hi = std::floor(a.x[0]);
  double lo = 0.0;
  if (hi == a.x[0]) {
    lo = std::floor(a.x[1]);
    return dd_shim::fast_two_sum(hi, lo);
  }
  return dd_real(hi, lo);
}

inline dd_real exp(const dd_real& a) { return dd_shim::exp(a); }
inline dd_real log(const dd_real& a) { return dd_shim::log(a); }

inline dd_real pow(const dd_real& a, const dd_real& b) {
  if (a.x[0] == 2.0 && a.x[1] == 0.0) return dd_shim::exp(dd_shim::mul(b, dd_shim::ln2()));
  return dd_shim::exp(dd_shim::mul(b, dd_shim::log(a)));
}

inline double to_double(const dd_real& a) { return a.x[0]; }

#endif /* GL_REF_SHIM_DD_REAL_H */
