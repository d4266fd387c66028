// gl_tables.cpp -- word sizes, weights and twiddles for one Lucas-Lehmer test.
//
// Double-double arithmetic after Dekker (1971) and Knuth (TAOCP 4.2.2): two-sum,
// two-product through fma, and renormalisation; the same published algorithms the
// QD library implements, which the reference uses for its weights
// (gpuLucas.cu:673-686).  exp() is a Taylor series on x/2^10 followed by ten
// squarings carried on expm1; sin/cos are Taylor series after an exact reduction to
// one octant by integer arithmetic on the angle's numerator.
#include "gl_tables.h"

#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace gl {
namespace {

struct DD {
  double hi, lo;
};

inline DD quick_two_sum(double a, double b) {
  double s = a + b;
  return {s, b - (s - a)};
}
inline DD two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
inline DD two_prod(double a, double b) {
  double p = a * b;
  return {p, std::fma(a, b, -p)};
}
inline DD dd(double a) { return {a, 0.0}; }
inline DD operator+(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  DD t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
inline DD operator-(DD a) { return {-a.hi, -a.lo}; }
inline DD operator-(DD a, DD b) { return a + (-b); }
inline DD operator*(DD a, DD b) {
  DD p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo;
  p.lo += a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
inline DD mul_d(DD a, double b) {
  DD p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
inline DD operator/(DD a, DD b) {
  double q1 = a.hi / b.hi;
  DD r = a - mul_d(b, q1);
  double q2 = r.hi / b.hi;
  r = r - mul_d(b, q2);
  double q3 = r.hi / b.hi;
  return quick_two_sum(q1, q2) + dd(q3);
}
inline double to_double(DD a) { return a.hi + a.lo; }

const DD kLn2 = {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
const DD kPi4 = {0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55};

// exp(x), 0 <= x < 1
DD exp_small(DD x) {
  DD y = {std::ldexp(x.hi, -10), std::ldexp(x.lo, -10)};
  DD term = y, sum = y;
  for (int k = 2; k <= 14; ++k) {
    term = (term * y) / dd((double)k);
    sum = sum + term;
  }
  for (int i = 0; i < 10; ++i) {
    DD two_s = {2.0 * sum.hi, 2.0 * sum.lo};
    sum = two_s + sum * sum;
  }
  return dd(1.0) + sum;
}

// sin, cos of (pi/4) num/den, 0 <= num <= den
void sincos_octant(int64_t num, int64_t den, DD* s, DD* c) {
  DD x = kPi4 * (dd((double)num) / dd((double)den));
  DD x2 = x * x;
  DD st = x, ss = x, ct = dd(1.0), cs = dd(1.0);
  for (int k = 1; k <= 14; ++k) {
    st = -((st * x2) / dd((double)((2 * k) * (2 * k + 1))));
    ss = ss + st;
    ct = -((ct * x2) / dd((double)((2 * k - 1) * (2 * k))));
    cs = cs + ct;
  }
  *s = ss;
  *c = cs;
}

inline int64_t ceil_div_pos(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& chunk) {
  unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = hw ? (int64_t)hw : 1;
  if (nt > 64) nt = 64;
  if (n < 4096 || nt == 1) {
    chunk(0, n);
    return;
  }
  if (nt > n / 1024) nt = n / 1024;
  std::vector<std::thread> th;
  th.reserve((size_t)nt);
  for (int64_t t = 0; t < nt; ++t) {
    const int64_t b = n * t / nt, e = n * (t + 1) / nt;
    th.emplace_back([&chunk, b, e] { chunk(b, e); });
  }
  for (auto& x : th) x.join();
}

int slice_depth(int p, int N) {
  if (N <= 0) return -1;
  int ratio = p / N;
  if (ratio >= 22) return -1;
  if (ratio >= 18) return 2;
  if (ratio >= 16) return 3;
  if (ratio >= 14) return 4;
  if (ratio >= 12) return 5;
  return 6;
}

int word_bits(int p, int N, int j) {
  return (int)(ceil_div_pos((int64_t)p * (j + 1), N) - ceil_div_pos((int64_t)p * j, N));
}

uint8_t word_flags(int p, int N, int j) {
  const int LO = p / N;
  uint8_t v = 0;
  for (int b = 0; b < 8; ++b) {
    const int k = ((j - b) % N + N) % N;
    v |= (uint8_t)((word_bits(p, N, k) != LO ? 1 : 0) << b);
  }
  return v;
}

void word_tables(int p, int N, std::vector<int32_t>& bits, std::vector<uint8_t>& flags) {
  bits.resize(N);
  flags.resize(N);
  for (int j = 0; j < N; ++j) bits[j] = (int32_t)word_bits(p, N, j);
  for (int j = 0; j < N; ++j) flags[j] = word_flags(p, N, j);
}

void weight_entry(int p, int N, int j, double inv_scale_den, double* A, double* Ainv) {
  // ceil(jp/N) - jp/N = r/N with r = ceil(jp/N)*N - jp, an exact integer
  const int64_t r = ceil_div_pos((int64_t)p * j, N) * N - (int64_t)p * j;
  const DD e = exp_small((dd((double)r) / dd((double)N)) * kLn2);
  *A = to_double(e);
  *Ainv = to_double((dd(1.0) / e) / dd(inv_scale_den));
}

void weight_tables(int p, int N, double inv_scale_den, std::vector<double>& A, std::vector<double>& Ainv) {
  A.resize(N);
  Ainv.resize(N);
  parallel_for(N, [&](int64_t b, int64_t e) {
    for (int64_t j = b; j < e; ++j) weight_entry(p, N, (int)j, inv_scale_den, &A[j], &Ainv[j]);
  });
}

namespace {
// cos and sin of 2 pi t / L in double-double
void cos_sin_dd(int64_t t, int64_t L, DD* C, DD* S) {
  t %= L;
  if (t < 0) t += L;
  int64_t u = 8 * t;
  int64_t o = u / L;
  int64_t r = u - o * L;
  DD s, c;
  if (o & 1) sincos_octant(L - r, L, &s, &c);
  else sincos_octant(r, L, &s, &c);
  switch (o) {
    case 0: *C = c; *S = s; break;
    case 1: *C = s; *S = c; break;
    case 2: *C = -s; *S = c; break;
    case 3: *C = -c; *S = s; break;
    case 4: *C = -c; *S = -s; break;
    case 5: *C = -s; *S = -c; break;
    case 6: *C = s; *S = -c; break;
    default: *C = c; *S = -s; break;
  }
}
}  // namespace

HostCplx twiddle(int64_t t, int64_t L) {
  DD C, S;
  cos_sin_dd(t, L, &C, &S);
  return {to_double(C), -to_double(S)};
}

HostCplx pair_coeff(int64_t k, int64_t M) {
  DD C, S;
  cos_sin_dd(k, M, &C, &S);
  // -(1 + cos - i sin)/4
  DD re = dd(1.0) + C;
  return {-0.25 * to_double(re), 0.25 * to_double(S)};
}

void twiddle_table(int64_t L, std::vector<HostCplx>& tw) {
  tw.resize(L);
  parallel_for(L, [&](int64_t b, int64_t e) {
    for (int64_t t = b; t < e; ++t) tw[t] = twiddle(t, L);
  });
}

int stage_values(int R) {
  switch (R) {
    case 2: return 1;
    case 3: return 4;
    case 4: return 4;
    case 8: return 8;
    case 16: return 8;
    default: return R - 1;
  }
}

namespace {
// w_L^t = cos(2 pi t/L) - i sin(2 pi t/L) = i^f rho (1 + i tau) with |tau| <= 1: f = 1 in
// the octants where |sin| >= |cos| (decided on the integer angle, so it is exact).  tau
// holds the stored value: tau for f = 0, -tau for f = 1.
struct RatioForm {
  DD rho, tau;
  int f;
};
RatioForm ratio_form(int64_t t, int64_t L) {
  t %= L;
  if (t < 0) t += L;
  DD C, S;
  cos_sin_dd(t, L, &C, &S);
  const DD re = C, im = -S;
  const int64_t o = (8 * t) / L;
  RatioForm r;
  if (o == 1 || o == 2 || o == 5 || o == 6) {
    r.f = 1;  // i rho (1 + i tau) = -rho tau + i rho: tau = -re/im, stored negated
    r.rho = im;
    r.tau = re / im;
  } else {
    r.f = 0;
    r.rho = re;
    r.tau = im / re;
  }
  return r;
}

// The stored doubles of one position of a twiddled radix-8, -4 or -3 stage (the ratio
// form the device butterflies read): w = w_L^e.
void ratio_values(int R, int64_t e, int64_t L, double* out) {
  RatioForm w[8];
  uint64_t fl = 0;
  for (int q = 1; q < R; ++q) {
    w[q] = ratio_form(e * q, L);
    fl |= (uint64_t)w[q].f << q;
  }
  double flags;
  std::memcpy(&flags, &fl, sizeof flags);
  auto rd = [](DD x) { return to_double(x); };
  auto ratio = [&](int a, int b) { return to_double(w[a].rho / w[b].rho); };
  if (R == 8) {
    DD c45, s45;
    sincos_octant(1, 1, &s45, &c45);  // cos(pi/4)
    const double v[16] = {rd(w[2].tau), rd(w[4].tau), rd(w[6].tau), flags,       rd(w[4].rho), ratio(6, 2),
                          rd(w[2].rho), ratio(5, 1),  rd(w[1].tau), rd(w[5].tau), rd(w[3].tau), rd(w[7].tau),
                          ratio(7, 3),  ratio(3, 1),  rd(w[1].rho), rd(w[1].rho * c45)};
    std::memcpy(out, v, sizeof v);
  } else if (R == 4) {
    const double v[8] = {rd(w[1].tau), rd(w[2].tau), rd(w[3].tau), flags, rd(w[2].rho), ratio(3, 1),
                         rd(w[1].rho), 0.0};
    std::memcpy(out, v, sizeof v);
  } else {
    DD c3, s3;
    cos_sin_dd(1, 3, &c3, &s3);  // sin(2 pi/3)
    const double v[8] = {rd(w[1].tau), rd(w[2].tau), ratio(2, 1), flags, rd(w[1].rho), 0.5 * rd(w[1].rho),
                         rd(w[1].rho * s3), 0.0};
    std::memcpy(out, v, sizeof v);
  }
}
}  // namespace

void stage_twiddles(int L, const std::vector<int>& radices, std::vector<HostCplx>& tw, int* off) {
  std::vector<HostCplx> base;
  twiddle_table(L, base);
  tw.assign(1, HostCplx{1.0, 0.0});
  int Ns = 1;
  for (size_t s = 0; s < radices.size(); ++s) {
    const int R = radices[s];
    off[s] = (int)tw.size();
    if (Ns > 1) {
      const int tws = L / (Ns * R);
      const int nv = stage_values(R);
      const size_t start = tw.size();
      tw.resize(start + (size_t)nv * Ns);
      for (int k = 0; k < Ns; ++k) {
        const int64_t e = (int64_t)k * tws;  // exponent of w = w_L^e
        if (R == 8 || R == 4 || R == 3) {
          double vals[16];
          ratio_values(R, e, L, vals);
          for (int v = 0; v < nv; ++v) tw[start + (size_t)v * Ns + k] = HostCplx{vals[2 * v], vals[2 * v + 1]};
        } else if (R & (R - 1)) {
          for (int q = 1; q < R; ++q) tw[start + (size_t)(q - 1) * Ns + k] = base[(e * q) % L];
        } else {
          int v = 0;
          for (int l = 1; (1 << l) <= R; ++l) {
            const int np = l == 1 ? 1 : (1 << (l - 2));
            for (int p = 0; p < np; ++p, ++v) {
              // w^(R/2^l) * W_(2^l)^p = w_L^(e R/2^l + p L/2^l)
              const int64_t idx = (e * (R >> l) + (int64_t)p * (L >> l)) % L;
              tw[start + (size_t)v * Ns + k] = base[idx];
            }
          }
        }
      }
    }
    Ns *= R;
  }
}

int radix_plan_into(int n, int max_radix, int* out, int cap) {
  if (n <= 0) return -1;
  int m = n, count = 0;
  const int radices[7] = {16, 8, 4, 2, 3, 5, 7};
  for (int q : radices) {
    if (q <= 16 && (q & (q - 1)) == 0 && q > max_radix) continue;  // power-of-two cap
    while (m % q == 0) {
      if (count == cap) return -1;
      out[count++] = q;
      m /= q;
    }
  }
  return m == 1 ? count : -1;
}

std::vector<int> radix_plan(int n, int max_radix) {
  int buf[64];
  const int count = radix_plan_into(n, max_radix, buf, 64);
  return count < 0 ? std::vector<int>() : std::vector<int>(buf, buf + count);
}

}  // namespace gl
