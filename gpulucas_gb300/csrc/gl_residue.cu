// gl_residue.cu -- end-of-run normalisation and Res64 on the device.
//
// The reference does this serially: addPseudoBalanced + rebalanceIrrIntSEQGPU, one
// thread walking all N words with a balanced carry (IrrBaseBalanced.cu:117-169, about 0.5 s per call
// at 26M-range exponents), then print_residue on the host borrows the digits
// non-negative and packs the low 64 bits (gpuLucas.cu:1288-1352).  Both walks are carry
// chains whose carry takes few values, so each word is a function from carry-in to
// carry-out and the chain is a prefix composition of those functions: a parallel
// carry-lookahead.
//
//   balanced pass:  x_j = digit[j] + hi[j-1]; t = x_j + c; carry +1 if t >= B/2,
//                   -1 if t < -B/2, else 0; out_j = t - carry*B; the carry out of the
//                   top word is added to out_0 (the reference's wrap, no further ripple)
//   canonical pass: t = out_j + c; carry = floor(t / B); y_j = t - carry*B in [0, B);
//                   the carry out of the top word re-enters word 0 (2^p == 1 mod
//                   2^p - 1): the carry into word 0 is the fixed point c0 = F(c0) of
//                   the whole chain F, which is F(0) (F is monotone with values in
//                   {-1, 0} on these inputs)
//
// Carries lie in {-1, 0, 1}; a carry function is stored as three 2-bit entries.
// Kernels: block functions (2048 words per block), one-block scan over the block
// functions, apply + next pass's block functions, scan, apply + zero flags.  The value
// is 0 mod 2^p - 1 exactly when the canonical digits are all 0 or all B_j - 1.
#include <cstdint>

#include "gl_internal.h"

namespace gl {
namespace {

constexpr int kResThreads = 256;
constexpr int kResItems = 8;
constexpr int kResWords = kResThreads * kResItems;
constexpr int kScanThreads = 1024;
constexpr uint32_t kFnId = 0u | (1u << 2) | (2u << 4);

__device__ __forceinline__ int fn_apply(uint32_t f, int c) { return (int)((f >> (2 * (c + 1))) & 3u) - 1; }
__device__ __forceinline__ uint32_t fn_make(int om, int o0, int op) {
  return (uint32_t)(om + 1) | ((uint32_t)(o0 + 1) << 2) | ((uint32_t)(op + 1) << 4);
}
// f first, then g
__device__ __forceinline__ uint32_t fn_then(uint32_t f, uint32_t g) {
  return fn_make(fn_apply(g, fn_apply(f, -1)), fn_apply(g, fn_apply(f, 0)), fn_apply(g, fn_apply(f, 1)));
}

__device__ __forceinline__ int bal_carry(int t, int bits) {
  const int half = 1 << (bits - 1);
  return t >= half ? 1 : (t < -half ? -1 : 0);
}
__device__ __forceinline__ int canon_carry(int t, int bits) { return t >> bits; }  // floor, |t| < 2^(bits+1)

__device__ __forceinline__ uint32_t bal_fn(int x, int bits) {
  return fn_make(bal_carry(x - 1, bits), bal_carry(x, bits), bal_carry(x + 1, bits));
}
__device__ __forceinline__ uint32_t canon_fn(int x, int bits) {
  return fn_make(canon_carry(x - 1, bits), canon_carry(x, bits), canon_carry(x + 1, bits));
}

// word j's bit count: LO, or LO + 1 when bit 0 of its flags byte is set
__device__ __forceinline__ int word_bits(const IterArgs& a, int j, bool colmajor_flags) {
  int idx = j;
  if (colmajor_flags) {
    const int m = j >> 1, m2 = m / a.W, m1 = m - m2 * a.W;
    idx = 2 * (m1 * a.H + m2) + (j & 1);
  }
  return a.LO + (int)(a.flags[idx] & 1u);
}

// Exclusive prefix (composition) of the block's thread functions, in thread order;
// *total receives the composition of all of them.  blockDim.x is a multiple of 32.
__device__ uint32_t block_scan_fn(uint32_t f, uint32_t* warp_tot, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t inc = f;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t g = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc = fn_then(g, inc);
  }
  uint32_t exc = __shfl_up_sync(0xffffffffu, inc, 1);
  if (lane == 0) exc = kFnId;
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nw ? warp_tot[lane] : kFnId;
    uint32_t winc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t g = __shfl_up_sync(0xffffffffu, winc, o);
      if (lane >= o) winc = fn_then(g, winc);
    }
    uint32_t wexc = __shfl_up_sync(0xffffffffu, winc, 1);
    if (lane == 0) wexc = kFnId;
    if (lane < nw) warp_tot[32 + lane] = wexc;
    if (lane == 31) warp_tot[64] = winc;
  }
  __syncthreads();
  const uint32_t pre = fn_then(warp_tot[32 + warp], exc);
  if (total) *total = warp_tot[64];
  __syncthreads();
  return pre;
}

// balanced-pass input word
__device__ __forceinline__ int bal_input(const IterArgs& a, int j) {
  return a.digit[j] + (int)a.hi[j == 0 ? a.N - 1 : j - 1];
}

// pass 1: block functions of the balanced pass
__global__ void __launch_bounds__(kResThreads) k_res_bal_fn(IterArgs a, bool cm, uint32_t* bf) {
  __shared__ uint32_t wt[65];
  const int j0 = blockIdx.x * kResWords + threadIdx.x * kResItems;
  uint32_t t = kFnId;
  for (int i = 0; i < kResItems; ++i) {
    const int j = j0 + i;
    if (j < a.N) t = fn_then(t, bal_fn(bal_input(a, j), word_bits(a, j, cm)));
  }
  uint32_t tot;
  block_scan_fn(t, wt, &tot);
  if (threadIdx.x == 0) bf[blockIdx.x] = tot;
}

// one block: exclusive prefix functions over `nb` block functions; scal[0] = carry into
// word 0 (0, or the fixed point F(0) when `wrap`), scal[1] = carry out of the top word
__global__ void __launch_bounds__(kScanThreads) k_res_scan(const uint32_t* bf, uint32_t* pf, int nb, bool wrap,
                                                           int* scal) {
  __shared__ uint32_t wt[65];
  uint32_t run = kFnId;
  for (int base = 0; base < nb; base += kScanThreads) {
    const int i = base + (int)threadIdx.x;
    const uint32_t f = i < nb ? bf[i] : kFnId;
    uint32_t tot;
    const uint32_t exc = block_scan_fn(f, wt, &tot);
    if (i < nb) pf[i] = fn_then(run, exc);
    run = fn_then(run, tot);
  }
  if (threadIdx.x == 0) {
    const int c0 = wrap ? fn_apply(run, 0) : 0;
    scal[0] = c0;
    scal[1] = fn_apply(run, c0);
  }
}

// pass 2: apply the balanced carries (out = balanced digits, the reference's
// rebalanced state), then the canonical pass's block functions of `out`
__global__ void __launch_bounds__(kResThreads) k_res_bal_apply(IterArgs a, bool cm, const uint32_t* pf,
                                                               const int* scal, int32_t* out, uint32_t* bf2) {
  __shared__ uint32_t wt[65];
  const int j0 = blockIdx.x * kResWords + threadIdx.x * kResItems;
  int x[kResItems], bits[kResItems];
  uint32_t t = kFnId;
#pragma unroll
  for (int i = 0; i < kResItems; ++i) {
    const int j = j0 + i;
    x[i] = 0;
    bits[i] = a.LO;
    if (j < a.N) {
      x[i] = bal_input(a, j);
      bits[i] = word_bits(a, j, cm);
      t = fn_then(t, bal_fn(x[i], bits[i]));
    }
  }
  const uint32_t pre = block_scan_fn(t, wt, nullptr);
  int c = fn_apply(pre, fn_apply(pf[blockIdx.x], scal[0]));
  uint32_t t2 = kFnId;
#pragma unroll
  for (int i = 0; i < kResItems; ++i) {
    const int j = j0 + i;
    if (j < a.N) {
      const int v = x[i] + c;
      const int co = bal_carry(v, bits[i]);
      int o = v - co * (1 << bits[i]);
      if (j == 0) o += scal[1];
      out[j] = o;
      c = co;
      t2 = fn_then(t2, canon_fn(o, bits[i]));
    }
  }
  uint32_t tot;
  block_scan_fn(t2, wt, &tot);
  if (threadIdx.x == 0) bf2[blockIdx.x] = tot;
}

// pass 3: canonical digits; head[j] for j < 64; flags bit 0: some digit != 0,
// bit 1: some digit != B_j - 1
__global__ void __launch_bounds__(kResThreads) k_res_canon_apply(IterArgs a, bool cm, const int32_t* out,
                                                                 const uint32_t* pf, const int* scal, int32_t* head,
                                                                 int* flags) {
  __shared__ uint32_t wt[65];
  __shared__ int sflags;
  if (threadIdx.x == 0) sflags = 0;
  const int j0 = blockIdx.x * kResWords + threadIdx.x * kResItems;
  int x[kResItems], bits[kResItems];
  uint32_t t = kFnId;
#pragma unroll
  for (int i = 0; i < kResItems; ++i) {
    const int j = j0 + i;
    x[i] = 0;
    bits[i] = a.LO;
    if (j < a.N) {
      x[i] = out[j];
      bits[i] = word_bits(a, j, cm);
      t = fn_then(t, canon_fn(x[i], bits[i]));
    }
  }
  const uint32_t pre = block_scan_fn(t, wt, nullptr);
  int c = fn_apply(pre, fn_apply(pf[blockIdx.x], scal[0]));
  int f = 0;
#pragma unroll
  for (int i = 0; i < kResItems; ++i) {
    const int j = j0 + i;
    if (j < a.N) {
      const int v = x[i] + c;
      const int co = canon_carry(v, bits[i]);
      const int y = v - co * (1 << bits[i]);
      c = co;
      if (y != 0) f |= 1;
      if (y != (1 << bits[i]) - 1) f |= 2;
      if (j < 64) head[j] = y;
    }
  }
  if (f) atomicOr(&sflags, f);
  __syncthreads();
  if (threadIdx.x == 0 && sflags) atomicOr(flags, sflags);
}

}  // namespace

size_t residue_scratch_bytes(int N) {
  const size_t nb = (size_t)(N + kResWords - 1) / kResWords;
  return 4 * nb * sizeof(uint32_t) + 64 * sizeof(int32_t) + 8 * sizeof(int);
}

// Scratch layout: bf, pf, bf2, pf2 (nb each), head[64], scal[4], scal2[2], flags.
cudaError_t launch_residue(const IterArgs& a, bool colmajor_flags, int32_t* balanced, void* scratch,
                           cudaStream_t s) {
  const int nb = (a.N + kResWords - 1) / kResWords;
  uint32_t* bf = static_cast<uint32_t*>(scratch);
  uint32_t* pf = bf + nb;
  uint32_t* bf2 = pf + nb;
  uint32_t* pf2 = bf2 + nb;
  int32_t* head = reinterpret_cast<int32_t*>(pf2 + nb);
  int* scal = head + 64;   // [0..1] balanced pass, [2..3] canonical pass
  int* flags = scal + 4;
  cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_res_bal_fn<<<nb, kResThreads, 0, s>>>(a, colmajor_flags, bf);
  k_res_scan<<<1, kScanThreads, 0, s>>>(bf, pf, nb, false, scal);
  k_res_bal_apply<<<nb, kResThreads, 0, s>>>(a, colmajor_flags, pf, scal, balanced, bf2);
  k_res_scan<<<1, kScanThreads, 0, s>>>(bf2, pf2, nb, true, scal + 2);
  k_res_canon_apply<<<nb, kResThreads, 0, s>>>(a, colmajor_flags, balanced, pf2, scal + 2, head, flags);
  return cudaGetLastError();
}

// offsets (in bytes) of head / scalars / flags inside the scratch, for the host read
size_t residue_head_offset(int N) {
  const size_t nb = (size_t)(N + kResWords - 1) / kResWords;
  return 4 * nb * sizeof(uint32_t);
}

}  // namespace gl
