// gl_kernels.cu -- sm_103a kernels of one Lucas-Lehmer iteration.
//
// Fused form (3 launches per iteration).  The N real words are packed as M = N/2
// complex points u[m] = x[2m] + i x[2m+1], arranged as an H x W array
// (m = m1 + W*m2).  The length-M DFT is done as four-step:
//   k_col_fwd : per column m1 (G columns per CTA): dice the previous products into
//               balanced digits + carries (llintToIrrBal<n>, IrrBaseBalanced.cu:52-110),
//               add the carry of the word below, weight (loadIntToDoubleIBDWT,
//               gpuLucas.cu:730-766), length-H DFT over m2, twiddle w_M^(m1 k2)
//   k_row_sq  : per row pair (k2, H-k2): length-W DFTs over m1, the real-signal split
//               and pointwise square (ComplexPointwiseSqr, gpuLucas.cu:647-665, for the
//               D2Z/Z2D pair of gpuLucas.cu:869-877), inverse length-W DFTs, twiddle
//               w_M^-(m1 k2)
//   k_col_inv : per column: inverse length-H DFT, unweight, subtract 2 at word 0, round
//               half-even to int64, round-off max (invDWTproductMinus2,
//               gpuLucas.cu:774-805)
// The products (int64) are the loop-carried state; the next k_col_fwd dices them.
//
// Plain form: one kernel per reference step, the FFT as one global-memory Stockham
// stage per launch (radix <= 4), state = (digit, hi) as in the reference.
#include "gl_device.cuh"
#include "gl_internal.h"

namespace gl {

static_assert(sizeof(DevCplx) == sizeof(cplx), "complex layout");

__device__ __forceinline__ cplx ld(const DevCplx* p) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return mk(v.x, v.y);
}
__device__ __forceinline__ cplx ldc(const DevCplx* p) {
  const double2 v = *reinterpret_cast<const double2*>(p);
  return mk(v.x, v.y);
}
__device__ __forceinline__ void st(DevCplx* p, cplx v) {
  *reinterpret_cast<double2*>(p) = make_double2(v.re, v.im);
}

// ---------------------------------------------------------------------------
// Stockham DIT stage in shared memory, out of place (src -> dst, one barrier).
// Butterfly j of a line reads src[j + q L/R], twiddles by w_L^((j mod Ns) q L/(Ns R)),
// does DFT_R and writes dst[(j - j mod Ns) R + j mod Ns + q Ns].  Each thread keeps
// one butterfly live at a time, so any block size works.
// ---------------------------------------------------------------------------
template <int R, int S>
__device__ __forceinline__ void stockham_stage(const cplx* __restrict__ src, cplx* __restrict__ dst, int nlines,
                                               int ls, int L, int Ns, const DevCplx* __restrict__ tw) {
  const int LR = L / R;
  const int nb = nlines * LR;
  const int tws = L / (Ns * R);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int l = b / LR;
    const int j = b - l * LR;
    const int k = j % Ns;
    const cplx* s = src + l * ls + j;
    cplx v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = s[q * LR];
    if (Ns > 1) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        const cplx w = ld(tw + k * q * tws);
        v[q] = (S < 0) ? cmul(v[q], w) : cmulc(v[q], w);
      }
    }
    dft<R, S>(v);
    cplx* d = dst + l * ls + (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) d[q * Ns] = v[q];
  }
  __syncthreads();
}

// Transforms nlines lines held in `a` (line stride ls) using `b` as the second buffer;
// returns the buffer that holds the result.
template <int S>
__device__ __forceinline__ cplx* line_fft(cplx* a, cplx* b, int nlines, int ls, const LinePlan& lp,
                                          const DevCplx* tw) {
  int Ns = 1;
  for (int s = 0; s < lp.nst; ++s) {
    switch (lp.radix[s]) {
      case 16: stockham_stage<16, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
      case 8: stockham_stage<8, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
      case 4: stockham_stage<4, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
      case 2: stockham_stage<2, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
      case 3: stockham_stage<3, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
      case 5: stockham_stage<5, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
      default: stockham_stage<7, S>(a, b, nlines, ls, lp.L, Ns, tw); break;
    }
    Ns *= lp.radix[s];
    cplx* t = a;
    a = b;
    b = t;
  }
  return a;
}

// Real-signal split and square for one frequency pair (k, M-k):
// e = U + conj(U'), o = -i (U - conj(U')), w = w_M^k;
// V_k = e^2 + w o^2 + 2i e o ;  V_{M-k} = conj(e^2 + w o^2) + 2i conj(e o).
// V is 4x the DFT of (z_even + i z_odd) of the squared real signal z.
__device__ __forceinline__ void pair_square(cplx u, cplx up, cplx w, cplx* vk, cplx* vkp) {
  const cplx e = mk(u.re + up.re, u.im - up.im);
  const cplx d = mk(u.re - up.re, u.im + up.im);
  const cplx o = mk(d.im, -d.re);
  const cplx e2 = mk(fma(e.re, e.re, -e.im * e.im), 2.0 * e.re * e.im);
  const cplx o2 = mk(fma(o.re, o.re, -o.im * o.im), 2.0 * o.re * o.im);
  const cplx q = cmul(o2, w);
  const cplx r = cmul(e, o);
  const double pr = e2.re + q.re, pi = e2.im + q.im;
  *vk = mk(fma(-2.0, r.im, pr), fma(2.0, r.re, pi));
  *vkp = mk(fma(2.0, r.im, pr), fma(2.0, r.re, -pi));
}

// ---------------------------------------------------------------------------
// Dicing helpers over the loop-carried products
// ---------------------------------------------------------------------------
struct WordSums {
  int v0, v1;  // digit + carry of the word below, for words j0 and j0+1
};

// words j0 = 2m, j0+1: digit sums of j0-1, j0, j0+1 from ll[j0-1-n .. j0+1]
__device__ __forceinline__ WordSums load_words(const IterArgs& a, int j0) {
  const long long* __restrict__ ll = a.ll;
  const unsigned char* __restrict__ fl = a.flags;
  const int N = a.N;
  auto at = [&](int j) -> long long { return __ldg(ll + (j < 0 ? j + N : j)); };
  const int jm = j0 == 0 ? N - 1 : j0 - 1;
  const uint32_t fm = __ldg(fl + jm), f0 = __ldg(fl + j0), f1 = __ldg(fl + j0 + 1);
  const long long sm1 = dice_sum(a.LO, a.n, fm, [&](int i) { return at(jm - i); });
  const long long s0 = dice_sum(a.LO, a.n, f0, [&](int i) { return at(j0 - i); });
  const long long s1 = dice_sum(a.LO, a.n, f1, [&](int i) { return at(j0 + 1 - i); });
  int dm, hm, d0, h0, d1, h1;
  balanced_split(sm1, a.LO + (int)(fm & 1), &dm, &hm);
  balanced_split(s0, a.LO + (int)(f0 & 1), &d0, &h0);
  balanced_split(s1, a.LO + (int)(f1 & 1), &d1, &h1);
  WordSums w;
  w.v0 = d0 + hm;
  w.v1 = d1 + h0;
  return w;
}

__device__ __forceinline__ WordSums load_state(const IterArgs& a, int j0) {
  const int jm = j0 == 0 ? a.N - 1 : j0 - 1;
  WordSums w;
  w.v0 = a.digit[j0] + (int)a.hi[jm];
  w.v1 = a.digit[j0 + 1] + (int)a.hi[j0];
  return w;
}

// ---------------------------------------------------------------------------
// Fused kernels
// ---------------------------------------------------------------------------
template <bool FROM_STATE>
__global__ void __launch_bounds__(kMaxThreads) k_col_fwd(IterArgs a) {
  extern __shared__ cplx smem[];
  const int G = a.G, H = a.H, W = a.W;
  const int c0 = blockIdx.x * G;
  const int ls = H;
  cplx* buf1 = smem + G * H;
  for (int idx = threadIdx.x; idx < G * H; idx += blockDim.x) {
    const int l = idx % G, m2 = idx / G;
    const int j0 = 2 * (c0 + l + W * m2);
    const WordSums w = FROM_STATE ? load_state(a, j0) : load_words(a, j0);
    const double x0 = __ldg(a.A + j0) * dbl_from_int(w.v0);
    const double x1 = __ldg(a.A + j0 + 1) * dbl_from_int(w.v1);
    smem[l * ls + m2] = mk(x0, x1);
  }
  __syncthreads();
  const cplx* res = line_fft<-1>(smem, buf1, G, ls, a.ph, a.twH);
  for (int idx = threadIdx.x; idx < G * H; idx += blockDim.x) {
    const int l = idx % G, k2 = idx / G;
    const int m1 = c0 + l;
    const cplx v = cmul(res[l * ls + k2], ld(a.twM + m1 * k2));
    st(a.Z + k2 * W + m1, v);
  }
}

__global__ void __launch_bounds__(kMaxThreads) k_row_sq(IterArgs a) {
  extern __shared__ cplx smem[];
  const int W = a.W, H = a.H;
  const int c = blockIdx.x;  // 0 .. H/2
  const int ra = c, rb = H - c;
  const bool self = (c == 0) || (2 * c == H);
  const int nl = self ? 1 : 2;
  cplx* buf1 = smem + 2 * W;
  for (int idx = threadIdx.x; idx < nl * W; idx += blockDim.x) {
    const int l = idx / W, k1 = idx - l * W;
    smem[idx] = ldc(a.Z + (l ? rb : ra) * W + k1);
  }
  __syncthreads();
  cplx* sp = line_fft<-1>(smem, buf1, nl, W, a.pw, a.twW);
  cplx* other = sp == smem ? buf1 : smem;
  if (!self) {
    for (int t = threadIdx.x; t < W; t += blockDim.x) {
      const int tp = W - 1 - t;
      cplx vk, vkp;
      pair_square(sp[t], sp[W + tp], ld(a.twM + ra + H * t), &vk, &vkp);
      sp[t] = vk;
      sp[W + tp] = vkp;
    }
  } else if (c == 0) {
    // row 0: frequency H*t pairs with H*((W - t) mod W)
    for (int t = threadIdx.x; t <= W / 2; t += blockDim.x) {
      const int tp = (W - t) % W;
      cplx vk, vkp;
      pair_square(sp[t], sp[tp], ld(a.twM + H * t), &vk, &vkp);
      sp[t] = vk;
      if (tp != t) sp[tp] = vkp;
    }
  } else {
    // row H/2: frequency H/2 + H*t pairs with H/2 + H*(W-1-t)
    for (int t = threadIdx.x; t < (W + 1) / 2; t += blockDim.x) {
      const int tp = W - 1 - t;
      cplx vk, vkp;
      pair_square(sp[t], sp[tp], ld(a.twM + ra + H * t), &vk, &vkp);
      sp[t] = vk;
      if (tp != t) sp[tp] = vkp;
    }
  }
  __syncthreads();
  const cplx* res = line_fft<+1>(sp, other, nl, W, a.pw, a.twW);
  for (int idx = threadIdx.x; idx < nl * W; idx += blockDim.x) {
    const int l = idx / W, m1 = idx - l * W;
    const int row = l ? rb : ra;
    const cplx v = cmulc(res[idx], ld(a.twM + m1 * row));
    st(a.Z + row * W + m1, v);
  }
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  return v;
}

// bits that product j can place into words j..j+n
__device__ __forceinline__ int slice_span(const IterArgs& a, int j) {
  int jn = j + a.n;
  if (jn >= a.N) jn -= a.N;
  const uint32_t f = __ldg(a.flags + jn);
  return (a.n + 1) * a.LO + __popc(f & ((1u << (a.n + 1)) - 1u));
}

__device__ __forceinline__ void finish_status(const IterArgs& a, unsigned long long emax, unsigned fl) {
  emax = warp_max_u64(emax);
  fl = __reduce_or_sync(0xffffffffu, fl);
  if ((threadIdx.x & 31) == 0) {
    if (emax) atomicMax(&a.status->maxerr64, emax);
    if (fl) atomicOr(&a.status->flags, fl);
  }
}

__device__ __forceinline__ long long unweight_word(const IterArgs& a, int j, double z, unsigned long long* emax,
                                                   unsigned* fl) {
  unsigned long long e;
  int big = 0;
  const double x = z * __ldg(a.Ainv + j);
  long long r = round_ll_bits(x, &e, &big);
  if (j == 0) r -= 2;  // the -2 of the LL step; exact on the rounded integer
  *emax = e > *emax ? e : *emax;
  const int span = slice_span(a, j);
  const unsigned long long mag = (unsigned long long)(r < 0 ? -r : r);
  if (big) *fl |= kStatusBig;
  if (span < 63 && (mag >> span) != 0ull) *fl |= kStatusSlice;
  return r;
}

__global__ void __launch_bounds__(kMaxThreads) k_col_inv(IterArgs a) {
  extern __shared__ cplx smem[];
  const int G = a.G, H = a.H, W = a.W;
  const int c0 = blockIdx.x * G;
  const int ls = H;
  cplx* buf1 = smem + G * H;
  for (int idx = threadIdx.x; idx < G * H; idx += blockDim.x) {
    const int l = idx % G, k2 = idx / G;
    smem[l * ls + k2] = ldc(a.Z + k2 * W + c0 + l);
  }
  __syncthreads();
  const cplx* res = line_fft<+1>(smem, buf1, G, ls, a.ph, a.twH);
  unsigned long long emax = 0;
  unsigned fl = 0;
  for (int idx = threadIdx.x; idx < G * H; idx += blockDim.x) {
    const int l = idx % G, m2 = idx / G;
    const int j0 = 2 * (c0 + l + W * m2);
    const cplx v = res[l * ls + m2];
    const long long r0 = unweight_word(a, j0, v.re, &emax, &fl);
    const long long r1 = unweight_word(a, j0 + 1, v.im, &emax, &fl);
    *reinterpret_cast<longlong2*>(a.ll + j0) = make_longlong2(r0, r1);
  }
  finish_status(a, emax, fl);
}

cudaError_t set_fused_smem_limits(const FusedGeom& g) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_col_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.sm_col))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.sm_col))) return e;
  if ((e = cudaFuncSetAttribute(k_col_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.sm_col))) return e;
  return cudaFuncSetAttribute(k_row_sq, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.sm_row);
}

cudaError_t launch_fused_iteration(const IterArgs& a, const FusedGeom& g, cudaStream_t s, bool from_state) {
  const int ncol = a.W / a.G;
  if (from_state) k_col_fwd<true><<<ncol, g.t_col, g.sm_col, s>>>(a);
  else k_col_fwd<false><<<ncol, g.t_col, g.sm_col, s>>>(a);
  k_row_sq<<<a.H / 2 + 1, g.t_row, g.sm_row, s>>>(a);
  k_col_inv<<<ncol, g.t_col, g.sm_col, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Plain form: one kernel per reference step
// ---------------------------------------------------------------------------

// loadIntToDoubleIBDWT (gpuLucas.cu:730-766): d[j] = A[j] (digit[j] + hi[j-1])
__global__ void k_plain_load(IterArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.N) return;
  const int v = a.digit[j] + (int)a.hi[j == 0 ? a.N - 1 : j - 1];
  reinterpret_cast<double*>(a.Z)[j] = a.A[j] * (double)v;
}

// one global-memory Stockham stage (same indexing as stockham_stage)
template <int R, int S>
__global__ void k_plain_stage(const DevCplx* __restrict__ x, DevCplx* __restrict__ y, int M, int Ns,
                              const DevCplx* __restrict__ twM) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int MR = M / R;
  if (j >= MR) return;
  const int k = j % Ns;
  const int tws = M / (Ns * R);
  cplx v[R];
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = ldc(x + j + q * MR);
  if (Ns > 1) {
#pragma unroll
    for (int q = 1; q < R; ++q) {
      const cplx w = ld(twM + k * q * tws);
      v[q] = (S < 0) ? cmul(v[q], w) : cmulc(v[q], w);
    }
  }
  dft<R, S>(v);
  DevCplx* dst = y + (j - k) * R + k;
#pragma unroll
  for (int q = 0; q < R; ++q) st(dst + q * Ns, v[q]);
}

// ComplexPointwiseSqr (gpuLucas.cu:647-665) with the real-signal split: pairs (k, M-k)
__global__ void k_plain_pair_square(DevCplx* Z, const DevCplx* __restrict__ twM, int M) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > M / 2) return;
  const int kp = k == 0 ? 0 : M - k;
  cplx vk, vkp;
  pair_square(ldc(Z + k), ldc(Z + kp), ld(twM + k), &vk, &vkp);
  st(Z + k, vk);
  if (kp != k) st(Z + kp, vkp);
}

// invDWTproductMinus2<1> (gpuLucas.cu:774-805) with the max round-off reduction
__global__ void k_plain_unweight(IterArgs a, const double* __restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long emax = 0;
  unsigned fl = 0;
  if (j < a.N) {
    double x = z[j] * a.Ainv[j];
    if (j == 0) x -= 2.0;
    const long long r = __double2ll_rn(x);
    const double e = fabs(x - rint(x));
    emax = (unsigned long long)ldexp(e, 64 - 1) << 1;  // e * 2^64 (e <= 0.5)
    if (fabs(x) >= 2251799813685248.0) fl |= kStatusBig;
    const int span = slice_span(a, j);
    const unsigned long long mag = (unsigned long long)(r < 0 ? -r : r);
    if (span < 63 && (mag >> span) != 0ull) fl |= kStatusSlice;
    a.ll[j] = r;
  }
  finish_status(a, emax, fl);
}

// llintToIrrBal<n> (IrrBaseBalanced.cu:52-110) over the whole signal
__global__ void k_dice(IterArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.N) return;
  const int N = a.N;
  const uint32_t f = a.flags[j];
  const long long s = dice_sum(a.LO, a.n, f, [&](int i) {
    const int k = j - i;
    return a.ll[k < 0 ? k + N : k];
  });
  int d, h;
  balanced_split(s, a.LO + (int)(f & 1), &d, &h);
  a.digit[j] = d;
  a.hi[j] = (signed char)h;
}

template <int S>
static void plain_fft(const IterArgs& a, const PlainGeom& g, DevCplx*& src, DevCplx*& dst, cudaStream_t s) {
  int Ns = 1;
  for (int st_ = 0; st_ < g.nst; ++st_) {
    const int R = g.radix[st_];
    const int nb = a.M / R;
    const int blocks = (nb + g.threads - 1) / g.threads;
    switch (R) {
      case 4: k_plain_stage<4, S><<<blocks, g.threads, 0, s>>>(src, dst, a.M, Ns, a.twM); break;
      case 2: k_plain_stage<2, S><<<blocks, g.threads, 0, s>>>(src, dst, a.M, Ns, a.twM); break;
      case 3: k_plain_stage<3, S><<<blocks, g.threads, 0, s>>>(src, dst, a.M, Ns, a.twM); break;
      case 5: k_plain_stage<5, S><<<blocks, g.threads, 0, s>>>(src, dst, a.M, Ns, a.twM); break;
      default: k_plain_stage<7, S><<<blocks, g.threads, 0, s>>>(src, dst, a.M, Ns, a.twM); break;
    }
    Ns *= R;
    DevCplx* t = src;
    src = dst;
    dst = t;
  }
}

cudaError_t launch_plain_iteration(const IterArgs& a, const PlainGeom& g, cudaStream_t s) {
  const int T = g.threads;
  k_plain_load<<<(a.N + T - 1) / T, T, 0, s>>>(a);
  DevCplx* src = a.Z;
  DevCplx* dst = a.Z2;
  plain_fft<-1>(a, g, src, dst, s);
  k_plain_pair_square<<<(a.M / 2 + 1 + T - 1) / T, T, 0, s>>>(src, a.twM, a.M);
  plain_fft<+1>(a, g, src, dst, s);
  k_plain_unweight<<<(a.N + T - 1) / T, T, 0, s>>>(a, reinterpret_cast<const double*>(src));
  k_dice<<<(a.N + T - 1) / T, T, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_dice(const IterArgs& a, cudaStream_t s) {
  k_dice<<<(a.N + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// loadValue4ToFFTarray (gpuLucas.cu:718-726) expressed in the loop-carried state:
// products ll = (4, 0, ..., 0), digits (4, 0, ..., 0), carries 0
__global__ void k_set_initial(IterArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.N) return;
  a.ll[j] = j == 0 ? 4 : 0;
  if (a.digit) a.digit[j] = j == 0 ? 4 : 0;
  if (a.hi) a.hi[j] = 0;
}

cudaError_t launch_set_initial(const IterArgs& a, int mode, cudaStream_t s) {
  (void)mode;
  k_set_initial<<<(a.N + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 throughput probe: 8 independent DFMA chains per thread, bounded loop.
// ---------------------------------------------------------------------------
__global__ void k_probe_dfma(double* out, long long iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (long long i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t probe_fp64(int blocks, int threads, long long iters, double* out, cudaStream_t s) {
  k_probe_dfma<<<blocks, threads, 0, s>>>(out, iters, 0.999999999, 1e-12);
  return cudaGetLastError();
}

}  // namespace gl
