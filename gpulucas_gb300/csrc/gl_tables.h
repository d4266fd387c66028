// gl_tables.h -- host precompute of a test's word sizes, IBDWT weights and FFT
// twiddles.  All floating point here is IEEE double / double-double with explicit
// fma and -ffp-contract=off, so the tables are bit-identical on x86_64 and aarch64.
#pragma once
#include <cstdint>
#include <vector>

#include <functional>

namespace gl {

// Run body(i) for i in [0, n) on the host's cores (std::thread, static chunks).
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& chunk);

struct HostCplx {
  double re, im;
};

// setSliceAndDice (gpuLucas.cu:323-343) extended to ratio 21; -1 when refused.
int slice_depth(int p, int N);

// bits[j] = ceil(p(j+1)/N) - ceil(pj/N) (computeBitsPerWord, gpuLucas.cu:688-694, in
// exact integer arithmetic); flags[j] bit i = word (j-i) mod N has LO+1 bits, i < 8
// (computeBitsPerWordVectors, gpuLucas.cu:700-714).
void word_tables(int p, int N, std::vector<int32_t>& bits, std::vector<uint8_t>& flags);
// One entry of each: bits[j] and flags[j] of word_tables (no containers).
int word_bits(int p, int N, int j);
uint8_t word_flags(int p, int N, int j);

// A[j] = 2^(ceil(jp/N) - jp/N) and Ainv[j] = 2^-(ceil(jp/N) - jp/N) * scale, computed in
// double-double and rounded once (computeWeightVectors, gpuLucas.cu:673-686, uses
// scale = 1/N; the fused kernels need 1/(2N)).
void weight_tables(int p, int N, double inv_scale_den, std::vector<double>& A, std::vector<double>& Ainv);

// One entry of weight_tables: A[j] and Ainv[j] (same rounding), no containers.
void weight_entry(int p, int N, int j, double inv_scale_den, double* A, double* Ainv);

// exp(-2 pi i t / L) for t in [0, L), correctly rounded from double-double.
void twiddle_table(int64_t L, std::vector<HostCplx>& tw);
HostCplx twiddle(int64_t t, int64_t L);

// Stage-ordered values of one Stockham line DFT of length L with the given radix
// sequence.  Stage s (span Ns, radix R, external twiddle w = w_L^(k L/(Ns R)) for
// butterfly position k < Ns) stores its 16-byte slots v-major at off[s] + v*Ns + k, so
// lanes with consecutive k read consecutive slots:
//  - R = 8, 4, 3: the ratio form of w^q = i^f rho_q (1 + i tau_q) (8, 4, 4 slots of two
//    doubles: tau, ratios of rho, flags; the order is the device butterflies', ratio_r8,
//    ratio_r4, ratio_r3 in gl_device.cuh);
//  - R = 2, 16: the layered radix-2 DIT needs, at level l = 1..log2 R, the values
//    w^(R/2^l) * W_(2^l)^p for p < max(1, 2^(l-2)) (the other half are the same times
//    +-i): v runs over (l=1,p=0), (l=2,p=0), (l=3,p=0..1), (l=4,p=0..3);
//  - R = 5, 7: w^q for q = 1..R-1.
// The first stage (Ns = 1) needs no table.  Returns the table (at least one entry)
// and fills off[] (offset of each stage).
void stage_twiddles(int L, const std::vector<int>& radices, std::vector<HostCplx>& tw, int* off);
// number of stored 16-byte slots per butterfly position for a stage of radix R
int stage_values(int R);

// -(1 + w_M^k)/4 from double-double cos/sin, rounded once: the coefficient of the
// real-signal square V_k = U_k^2 + c_k (U_k - conj(U_{M-k}))^2.
HostCplx pair_coeff(int64_t k, int64_t M);

// factor n into the allowed radices (16, 8, 4, 2, 3, 5, 7; powers of two up to
// max_radix), largest power of two first, then 3, 5, 7; empty if n has another prime
// factor.
std::vector<int> radix_plan(int n, int max_radix);
// The same into out[0..cap): returns the number of stages, or -1 if n has another prime
// factor or needs more than cap stages.
int radix_plan_into(int n, int max_radix, int* out, int cap);

}  // namespace gl
