/* gpulucas.hpp -- C++ conveniences over the C ABI of gpulucas.h.
 *
 * llintToBalInt<n>: the carry semantics of the reference's llintToIrrBal<n>
 * (IrrBaseBalanced.cu:52-110, named llintToBalInt<n> in README:80-86 and gpuLucas.cu:59)
 * as a host/device inline, for callers and tests that need the digit state of a
 * product vector without a plan.  Word j of the result takes from the rounded products
 * of words j, j-1, ..., j-n (cyclically) the bits that belong to it:
 *
 *   sum_j = sum_{i=0..n} sgn(ll[j-i]) * ((|ll[j-i]| >> shift_i) & (2^bits_j - 1)),
 *   shift_0 = 0, shift_i = bits_{j-1} + ... + bits_{j-i},
 *
 * then splits it balanced: hi_j = the carry (int8), digit_j = sum_j - hi_j * 2^bits_j
 * with digit_j in [-2^(bits_j - 1), 2^(bits_j - 1)).  The carry hi_j is added to word
 * j + 1 at the next load (loadIntToDoubleIBDWT, gpuLucas.cu:730-766).  The word sizes
 * are bits_j = ceil(p (j+1) / N) - ceil(p j / N) (computeBitsPerWord, gpuLucas.cu:688-694,
 * in exact integer arithmetic).
 *
 * The library's kernels implement the same arithmetic (they read the word sizes from
 * a flags table instead); a test can compare the two on any product vector through
 * gl_set_products + gl_get_carry_state.
 */
#ifndef GPULUCAS_HPP
#define GPULUCAS_HPP

#include <cstdint>

#include "gpulucas.h"

#if defined(__CUDACC__)
#define GPULUCAS_HD __host__ __device__ inline
#else
#define GPULUCAS_HD inline
#endif

namespace gpulucas {

/* bits of word j of 2^p - 1 at FFT length N */
GPULUCAS_HD int word_bits(int p, int N, int j) {
  const int64_t hi = ((int64_t)p * (j + 1) + N - 1) / N;
  const int64_t lo = ((int64_t)p * j + N - 1) / N;
  return (int)(hi - lo);
}

/* Digit and carry of word j from the products ll[0..N) (carry depth n, as
 * setSliceAndDice(p, N) returns it). */
template <int n>
GPULUCAS_HD void llintToBalInt(const int64_t* ll, int p, int N, int j, int32_t* digit, int8_t* hi) {
  const int bits = word_bits(p, N, j);
  const int64_t mask = ((int64_t)1 << bits) - 1;
  int64_t v = ll[j];
  int64_t sum = v < 0 ? -((-v) & mask) : (v & mask);
  int shift = 0;
  for (int i = 1; i <= n; ++i) {
    int k = j - i;
    if (k < 0) k += N;
    shift += word_bits(p, N, k);
    if (shift >= 63) break;  // nothing of a 63-bit magnitude lies this high
    const int64_t w = ll[k];
    sum += w < 0 ? -(((-w) >> shift) & mask) : ((w >> shift) & mask);
  }
  const int64_t half = (int64_t)1 << (bits - 1);
  int64_t h = 0;
  if (sum < -half) h = -((-sum + half) >> bits);
  else if (sum >= half) h = (sum + half) >> bits;
  *digit = (int32_t)(sum - h * ((int64_t)1 << bits));
  *hi = (int8_t)h;
}

/* All N words; n is the carry depth (1..4). */
inline int llintToBalInt(int n, const int64_t* ll, int p, int N, int32_t* digit, int8_t* hi) {
  for (int j = 0; j < N; ++j) {
    switch (n) {
      case 1: llintToBalInt<1>(ll, p, N, j, digit + j, hi + j); break;
      case 2: llintToBalInt<2>(ll, p, N, j, digit + j, hi + j); break;
      case 3: llintToBalInt<3>(ll, p, N, j, digit + j, hi + j); break;
      case 4: llintToBalInt<4>(ll, p, N, j, digit + j, hi + j); break;
      default: return GL_ERR_ARG;
    }
  }
  return GL_OK;
}

}  // namespace gpulucas

#undef GPULUCAS_HD
#endif /* GPULUCAS_HPP */
