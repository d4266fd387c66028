// gl_hostcheck.cu -- the device arithmetic helpers (small DFTs, integer-domain
// rounding and conversion, dicing) compiled for the host, so the CPU test suite can
// check them against numpy and the oracle without a GPU.  Not used by the product.
#include <cstdint>

#include "gl_device.cuh"

using namespace gl;

template <int S>
static void run_dft(int R, cplx* x) {
  switch (R) {
    case 2: dft<2, S>(x); break;
    case 3: dft<3, S>(x); break;
    case 4: dft<4, S>(x); break;
    case 5: dft<5, S>(x); break;
    case 7: dft<7, S>(x); break;
    case 8: dft<8, S>(x); break;
    case 16: dft<16, S>(x); break;
    default: break;
  }
}

extern "C" {

// in-place DFT of R interleaved complex doubles; sign -1 forward, +1 inverse
int hc_dft(int R, int sign, double* xy) {
  if (R != 2 && R != 3 && R != 4 && R != 5 && R != 7 && R != 8 && R != 16) return -1;
  cplx* x = reinterpret_cast<cplx*>(xy);
  if (sign < 0) run_dft<-1>(R, x);
  else run_dft<1>(R, x);
  return 0;
}

long long hc_round(double x, unsigned long long* err64, int* big) {
  *big = 0;
  return round_ll_bits(x, err64, big);
}

double hc_dbl_from_int(int v) { return dbl_from_int(v); }

// dice one word j from products ll (cyclic, length N) with flags
struct CyclicProducts {
  const long long* ll;
  int N, j;
  __host__ __device__ long long operator()(int i) const {
    const int k = j - i;
    return ll[k < 0 ? k + N : k];
  }
};

long long hc_dice_sum(int LO, int n, unsigned f, const long long* ll, int N, int j) {
  return dice_sum(LO, n, f, CyclicProducts{ll, N, j});
}

void hc_balanced_split(long long sum, int bits, int* digit, int* hi) { balanced_split(sum, bits, digit, hi); }

}  // extern "C"

// The product's host tables (gl_tables.cpp), for pinning against the golden values.
#include <vector>

#include "gl_tables.h"

extern "C" {

void hc_weights(int p, int N, double* A, double* Ainv) {
  std::vector<double> a, ai;
  gl::weight_tables(p, N, (double)N, a, ai);
  for (int j = 0; j < N; ++j) {
    A[j] = a[j];
    Ainv[j] = ai[j];
  }
}

void hc_twiddles(int L, double* re, double* im) {
  for (int t = 0; t < L; ++t) {
    gl::HostCplx w = gl::twiddle(t, L);
    re[t] = w.re;
    im[t] = w.im;
  }
}

void hc_word_tables(int p, int N, int* bits, unsigned char* flags) {
  std::vector<int32_t> b;
  std::vector<uint8_t> f;
  gl::word_tables(p, N, b, f);
  for (int j = 0; j < N; ++j) {
    bits[j] = b[j];
    flags[j] = f[j];
  }
}

}  // extern "C"

extern "C" {

// layered radix-2^k DIT of R points (interleaved complex), external-twiddle values
// tv (R/2 complex, or 1 for R = 2) when with_tw, else the constant first-stage form
int hc_layered(int R, int sign, int with_tw, const double* tv, double* xy) {
  cplx* x = reinterpret_cast<cplx*>(xy);
  const cplx* t = reinterpret_cast<const cplx*>(tv);
  if (sign < 0) {
    switch (R) {
      case 2: with_tw ? layered_dit<2, -1, true>(x, t) : layered_dit<2, -1, false>(x, t); break;
      case 4: with_tw ? layered_dit<4, -1, true>(x, t) : layered_dit<4, -1, false>(x, t); break;
      case 8: with_tw ? layered_dit<8, -1, true>(x, t) : layered_dit<8, -1, false>(x, t); break;
      case 16: with_tw ? layered_dit<16, -1, true>(x, t) : layered_dit<16, -1, false>(x, t); break;
      default: return -1;
    }
  } else {
    switch (R) {
      case 2: with_tw ? layered_dit<2, 1, true>(x, t) : layered_dit<2, 1, false>(x, t); break;
      case 4: with_tw ? layered_dit<4, 1, true>(x, t) : layered_dit<4, 1, false>(x, t); break;
      case 8: with_tw ? layered_dit<8, 1, true>(x, t) : layered_dit<8, 1, false>(x, t); break;
      case 16: with_tw ? layered_dit<16, 1, true>(x, t) : layered_dit<16, 1, false>(x, t); break;
      default: return -1;
    }
  }
  return 0;
}

}  // extern "C"

extern "C" {

// the product's stage-ordered twiddle table for a line of length L (returns the size;
// out may be NULL to query it), offsets per stage into off
int hc_stage_twiddles(int L, const int* radices, int nst, double* out, int* off) {
  std::vector<int> r(radices, radices + nst);
  std::vector<gl::HostCplx> tw;
  gl::stage_twiddles(L, r, tw, off);
  if (out)
    for (size_t i = 0; i < tw.size(); ++i) {
      out[2 * i] = tw[i].re;
      out[2 * i + 1] = tw[i].im;
    }
  return (int)tw.size();
}

void hc_pair_coeff(int k, int M, double* c) {
  gl::HostCplx v = gl::pair_coeff(k, M);
  c[0] = v.re;
  c[1] = v.im;
}

}  // extern "C"

// One line DFT of length L with the given radices, run on the host through the device
// butterfly (stage_dft) and the product's stage-ordered table, in the Stockham order of
// the kernels' shared-memory stages (without the padding).  sign -1 forward, +1 inverse
// (unscaled).  Returns 0, or -1 for an unsupported radix.
namespace {
struct TableSlot {
  const cplx* tw;
  int Ns, k;
  __host__ __device__ cplx operator()(int i) const { return tw[(size_t)i * Ns + k]; }
};

template <int S>
int host_stage(int R, const cplx* src, cplx* dst, int L, int Ns, const cplx* tw) {
  const int LR = L / R;
  for (int j = 0; j < LR; ++j) {
    const int k = j % Ns;
    cplx v[16];
    for (int q = 0; q < R; ++q) v[q] = src[j + q * LR];
    const TableSlot slot{tw, Ns, k};
    const bool t = Ns > 1;
    switch (R) {
      case 2: stage_dft<2, S>(v, t, slot); break;
      case 3: stage_dft<3, S>(v, t, slot); break;
      case 4: stage_dft<4, S>(v, t, slot); break;
      case 5: stage_dft<5, S>(v, t, slot); break;
      case 7: stage_dft<7, S>(v, t, slot); break;
      case 8: stage_dft<8, S>(v, t, slot); break;
      case 16: stage_dft<16, S>(v, t, slot); break;
      default: return -1;
    }
    const int base = (j - k) * R + k;
    for (int q = 0; q < R; ++q) dst[base + q * Ns] = v[q];
  }
  return 0;
}
}  // namespace

extern "C" int hc_line_fft(int L, const int* radices, int nst, int sign, double* xy) {
  std::vector<int> r(radices, radices + nst);
  std::vector<gl::HostCplx> tw;
  int off[16];
  if (nst > 16) return -1;
  gl::stage_twiddles(L, r, tw, off);
  std::vector<cplx> a(reinterpret_cast<cplx*>(xy), reinterpret_cast<cplx*>(xy) + L), b((size_t)L);
  const cplx* t = reinterpret_cast<const cplx*>(tw.data());
  int Ns = 1;
  for (int s = 0; s < nst; ++s) {
    const int st = sign < 0 ? host_stage<-1>(r[s], a.data(), b.data(), L, Ns, t + off[s])
                            : host_stage<1>(r[s], a.data(), b.data(), L, Ns, t + off[s]);
    if (st) return st;
    Ns *= r[s];
    a.swap(b);
  }
  for (int i = 0; i < L; ++i) {
    xy[2 * i] = a[i].re;
    xy[2 * i + 1] = a[i].im;
  }
  return 0;
}
