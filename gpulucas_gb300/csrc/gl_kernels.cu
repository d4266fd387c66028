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
//               w_M^-(m1 k2), stored column-major into a second work array so that the
//               inverse column pass reads its column contiguously (the transposing
//               accesses are stores, which do not stall the issuing warp)
//   k_col_inv : per column: inverse length-H DFT, unweight, subtract 2 at word 0, round
//               half-even to int64, round-off max (invDWTproductMinus2,
//               gpuLucas.cu:774-805)
// The products (int64) are the loop-carried state; the next k_col_fwd dices them.
//
// Plain form: one kernel per reference step, the FFT as one global-memory Stockham
// stage per launch (radix <= 4), state = (digit, hi) as in the reference.
#include <cooperative_groups.h>

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
// a twiddle from the global table (read-only path) or from a shared-memory copy
__device__ __forceinline__ cplx tw_at(const DevCplx* p) { return ld(p); }
__device__ __forceinline__ cplx tw_at(const cplx* p) { return *p; }

// ---------------------------------------------------------------------------
// Bulk copies global -> shared (cp.async.bulk, the TMA's untiled form) completing on an
// mbarrier.  Every wait is bounded: after kWaitTries polls (each may suspend the thread
// for a while) it reports failure and the caller returns with kStatusTimeout.
// ---------------------------------------------------------------------------
constexpr int kWaitTries = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals = 1) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one thread: expect `bytes` on the barrier and start the copy (16-byte aligned
// addresses, bytes a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int tries = kWaitTries) {
  for (int i = 0; i < tries; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Shared-memory line FFTs.  Element i of a line sits at pad(i) = i + i/16: the
// Stockham writes of a stage with span 1 go to stride-R addresses, which without
// the pad would all fall into one bank group.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }

// Stockham DIT stage, out of place (src -> dst, one barrier).  Butterfly j of a
// line reads x[j + q L/R], applies the external twiddle w^q with
// w = w_L^((j mod Ns) L/(Ns R)), does DFT_R and writes x[(j - j mod Ns) R + j mod Ns +
// p Ns].  The butterfly itself is stage_dft (gl_device.cuh); its stored values for
// position k are the slots off + v Ns + k of the stage-ordered table, so lanes with
// consecutive k read consecutive slots.
template <int R, int S, typename TW>
__device__ __forceinline__ void stockham_stage(const cplx* __restrict__ src, cplx* __restrict__ dst, int nlines,
                                               int ls, int L, int Ns, const TW* __restrict__ tw) {
  const int LR = L / R;
  const int nb = nlines * LR;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int l = b / LR;
    const int j = b - l * LR;
    const int k = j % Ns;
    const cplx* s = src + l * ls;
    cplx v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = s[pad(j + q * LR)];
    const TW* tk = tw + k;
    stage_dft<R, S>(v, Ns > 1, [&](int i) { return tw_at(tk + (size_t)i * Ns); });
    cplx* d = dst + l * ls;
    const int base = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) d[pad(base + q * Ns)] = v[q];
  }
  __syncthreads();
}

// Transforms nlines lines held in `a` (line stride ls) using `b` as the second buffer;
// returns the buffer that holds the result.  R43: the plan has only radices 4, 3 and 2, and
// only those stages are compiled (a kernel's registers are set by its largest stage).
template <int S, bool R43 = false, typename TW>
__device__ __forceinline__ cplx* line_fft(cplx* a, cplx* b, int nlines, int ls, const LinePlan& lp,
                                          const TW* tw) {
  int Ns = 1;
  for (int s = 0; s < lp.nst; ++s) {
    const TW* st = tw + lp.off[s];
    static_assert(kMaxRadix == 8, "line plans use radices 2, 4, 8, 3, 5, 7");
    if (R43) {
      switch (lp.radix[s]) {
        case 4: stockham_stage<4, S>(a, b, nlines, ls, lp.L, Ns, st); break;
        case 2: stockham_stage<2, S>(a, b, nlines, ls, lp.L, Ns, st); break;
        default: stockham_stage<3, S>(a, b, nlines, ls, lp.L, Ns, st); break;
      }
    } else switch (lp.radix[s]) {
      case 8: stockham_stage<8, S>(a, b, nlines, ls, lp.L, Ns, st); break;
      case 4: stockham_stage<4, S>(a, b, nlines, ls, lp.L, Ns, st); break;
      case 2: stockham_stage<2, S>(a, b, nlines, ls, lp.L, Ns, st); break;
      case 3: stockham_stage<3, S>(a, b, nlines, ls, lp.L, Ns, st); break;
      case 5: stockham_stage<5, S>(a, b, nlines, ls, lp.L, Ns, st); break;
      default: stockham_stage<7, S>(a, b, nlines, ls, lp.L, Ns, st); break;
    }
    Ns *= lp.radix[s];
    cplx* t = a;
    a = b;
    b = t;
  }
  return a;
}

// The threads that run one line DFT: thread g.tid of g.n, synchronised by barrier g.bar
// (0: the whole block, __syncthreads; 1, 2: a named barrier of the g.n threads of one half
// of a block whose two halves work on different columns).
struct Grp {
  int tid, n, bar;
  __device__ __forceinline__ void sync() const {
    // immediate barrier numbers, so the kernel reserves barriers 0-2 only
    if (bar == 0) __syncthreads();
    else if (bar == 1) asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory");
    else asm volatile("bar.sync 2, %0;" ::"r"(n) : "memory");
  }
};
__device__ __forceinline__ Grp whole_block() { return Grp{(int)threadIdx.x, (int)blockDim.x, 0}; }

// In-place variant (one buffer, two barriers per stage): every thread first reads the
// inputs of all its butterflies of the stage into registers (at most 8 points: one radix-8
// butterfly, two radix-4, four radix-2, one odd-radix), then, after the barrier, computes
// and writes them back.  Half the shared memory of the ping-pong form, so more CTAs fit
// on an SM; usable when every stage has at most that many butterflies per thread.
template <int R>
__host__ __device__ constexpr int ip_butterflies() {
  return (R & (R - 1)) == 0 ? 8 / R : 1;
}

template <int R, int S, typename TW>
__device__ __forceinline__ void stockham_stage_ip(cplx* __restrict__ buf, int nlines, int ls, int L, int Ns,
                                                  const TW* __restrict__ tw, const Grp& g) {
  constexpr int B = ip_butterflies<R>();
  const int LR = L / R;
  const int nb = nlines * LR;
  cplx held[B * R];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int b = g.tid + i * g.n;
    const int bb = b < nb ? b : 0;  // a thread without this butterfly reads a valid slot
    const int l = bb / LR;
    const int j = bb - l * LR;
    const cplx* s = buf + l * ls;
#pragma unroll
    for (int q = 0; q < R; ++q) held[i * R + q] = s[pad(j + q * LR)];
  }
  g.sync();
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int b = g.tid + i * g.n;
    if (b < nb) {
      const int l = b / LR;
      const int j = b - l * LR;
      const int k = j % Ns;
      cplx v[R];
#pragma unroll
      for (int q = 0; q < R; ++q) v[q] = held[i * R + q];
      const TW* tk = tw + k;
      stage_dft<R, S>(v, Ns > 1, [&](int t) { return tw_at(tk + (size_t)t * Ns); });
      cplx* d = buf + l * ls;
      const int base = (j - k) * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) d[pad(base + q * Ns)] = v[q];
    }
  }
  g.sync();
}

template <int S, typename TW>
__device__ __forceinline__ cplx* line_fft_ip(cplx* a, int nlines, int ls, const LinePlan& lp, const TW* tw,
                                             const Grp& g) {
  int Ns = 1;
  for (int s = 0; s < lp.nst; ++s) {
    const TW* st = tw + lp.off[s];
    switch (lp.radix[s]) {
      case 8: stockham_stage_ip<8, S>(a, nlines, ls, lp.L, Ns, st, g); break;
      case 4: stockham_stage_ip<4, S>(a, nlines, ls, lp.L, Ns, st, g); break;
      case 2: stockham_stage_ip<2, S>(a, nlines, ls, lp.L, Ns, st, g); break;
      case 3: stockham_stage_ip<3, S>(a, nlines, ls, lp.L, Ns, st, g); break;
      case 5: stockham_stage_ip<5, S>(a, nlines, ls, lp.L, Ns, st, g); break;
      default: stockham_stage_ip<7, S>(a, nlines, ls, lp.L, Ns, st, g); break;
    }
    Ns *= lp.radix[s];
  }
  return a;
}

// Real-signal split and square for one frequency pair (k, M-k).  With U the DFT of
// u[m] = x[2m] + i x[2m+1], E/O the DFTs of the even/odd words, E + iO = U_k, so the
// DFT of (z_even + i z_odd) of the squared signal is
//   V_k = E^2 + w O^2 + 2i E O = U_k^2 + (1 + w) O^2 = U_k^2 + c_k D^2,
// D = U_k - conj(U_{M-k}), c_k = -(1 + w_M^k)/4 (from the table), and
//   V_{M-k} = U_{M-k}^2 + conj(c_k D^2).   19 FP64 instructions per pair.
__device__ __forceinline__ void pair_square(cplx u, cplx up, cplx c, cplx* vk, cplx* vkp) {
  const cplx d = mk(u.re - up.re, u.im + up.im);
  const cplx d2 = mk(fma(d.re, d.re, -d.im * d.im), 2.0 * d.re * d.im);
  const cplx pc = cmul(c, d2);
  *vk = mk(fma(u.re, u.re, fma(-u.im, u.im, pc.re)), fma(2.0 * u.re, u.im, pc.im));
  *vkp = mk(fma(up.re, up.re, fma(-up.im, up.im, pc.re)), fma(2.0 * up.re, up.im, -pc.im));
}

// column-major position of natural word j (fused form layout)
__device__ __forceinline__ int colmajor(const IterArgs& a, int j) {
  const int m = j >> 1;
  const int m2 = m / a.W;
  const int m1 = m - m2 * a.W;
  return 2 * (m1 * a.H + m2) + (j & 1);
}

// ---------------------------------------------------------------------------
// Fused kernels (one column / one row pair per CTA)
// ---------------------------------------------------------------------------

// Column pass, forward.  NC = carry depth n of llintToIrrBal<n>.  For words
// j0 = 2m, j0+1 the digit sums of j0-1, j0, j0+1 need the products of words
// j0-1-NC .. j0+1: P[k] = product of word j0+1-k, k = 0 .. NC+2.  Words j0+1-2d and
// j0-2d are the two words of point m-d, column m1-d of the same row (the previous row,
// from the last columns, when m1 < d), adjacent in the column-major layout: one 16-byte
// load per point, and no division to find it.
// Loads column m1 into buf (threads tid, tid + nth, ...): dice the previous products into
// balanced digits and carries, add the carry of the word below, weight.
template <bool FROM_STATE, int NC>
__device__ __forceinline__ void col_fwd_load(const IterArgs& a, const int m1, cplx* buf, int tid, int nth) {
  const int H = a.H, W = a.W, N = a.N, LO = a.LO;
  constexpr int D = (NC + 2) / 2;  // points m-1 .. m-D hold the words j0-1 .. j0+1-(NC+2)
  // two points' loads in flight per thread (C3: 0.3038 -> 0.3016 ms per iteration); four,
  // or unrolling the passes' other per-point loops as well, spills registers
#pragma unroll 2
  for (int m2 = tid; m2 < H; m2 += nth) {
    const int s0 = 2 * (m1 * H + m2);
    int v0, v1;
    if (FROM_STATE) {
      const int j0 = 2 * (m1 + W * m2);
      v0 = a.digit[j0] + (int)a.hi[j0 == 0 ? N - 1 : j0 - 1];
      v1 = a.digit[j0 + 1] + (int)a.hi[j0];
    } else {
      long long P[NC + 3];
      const longlong2 own = __ldg(reinterpret_cast<const longlong2*>(a.ll + s0));
      P[0] = own.y;
      P[1] = own.x;
      uint32_t fm = 0;  // flags of word j0-1 (the upper word of point m-1)
#pragma unroll
      for (int d = 1; d <= D; ++d) {
        int c = m1 - d, r = m2;
        if (c < 0) {  // one wrap suffices: layouts have W >= 4 >= D
          c += W;
          r = r == 0 ? H - 1 : r - 1;
        }
        const int sd = 2 * (c * H + r);
        if (d == 1) fm = __ldg(a.flags + sd + 1);
        if (2 * d + 1 < NC + 3) {
          const longlong2 v = __ldg(reinterpret_cast<const longlong2*>(a.ll + sd));
          P[2 * d] = v.y;
          P[2 * d + 1] = v.x;
        } else {  // only the upper word of the farthest point
          P[2 * d] = __ldg(a.ll + sd + 1);
        }
      }
      const uint32_t f0 = __ldg(a.flags + s0), f1 = __ldg(a.flags + s0 + 1);
      auto dice_at = [&](uint32_t f, int off) {
        const long long mask = (1ll << (LO + (int)(f & 1))) - 1;
        const long long v = P[off];
        long long sum = v < 0 ? -((-v) & mask) : (v & mask);
        int shift = 0;
#pragma unroll
        for (int i = 1; i <= NC; ++i) {
          shift += LO + (int)((f >> i) & 1);
          const long long w = P[off + i];
          sum += shift >= 63 ? 0 : (w < 0 ? -(((-w) >> shift) & mask) : ((w >> shift) & mask));
        }
        return sum;
      };
      const long long sw1 = dice_at(f1, 0), sw0 = dice_at(f0, 1), sm1 = dice_at(fm, 2);
      int dm, hm, d0, h0, d1, h1;
      balanced_split(sm1, LO + (int)(fm & 1), &dm, &hm);
      balanced_split(sw0, LO + (int)(f0 & 1), &d0, &h0);
      balanced_split(sw1, LO + (int)(f1 & 1), &d1, &h1);
      v0 = d0 + hm;
      v1 = d1 + h0;
    }
    const double2 A = __ldg(reinterpret_cast<const double2*>(a.A + s0));
    buf[pad(m2)] = mk(A.x * dbl_from_int(v0), A.y * dbl_from_int(v1));
  }
}

// twiddle w_M^(m1 k2) and store column m1 into row k2 of Z
__device__ __forceinline__ void col_fwd_store(const IterArgs& a, const int m1, const cplx* res, int tid, int nth) {
  const int H = a.H, W = a.W;
  const DevCplx* tw = a.twK1 + (size_t)m1 * H;
  for (int k2 = tid; k2 < H; k2 += nth) st(a.Z + (size_t)k2 * W + m1, cmul(res[pad(k2)], ld(tw + k2)));
}

template <bool FROM_STATE, int NC, bool IP = false>
__device__ __forceinline__ void col_fwd_body(const IterArgs& a, const int m1) {
  extern __shared__ cplx smem[];
  const int ls = a.ls_col;
  col_fwd_load<FROM_STATE, NC>(a, m1, smem, threadIdx.x, blockDim.x);
  __syncthreads();
  const cplx* res = IP ? line_fft_ip<-1>(smem, 1, ls, a.ph, a.twH, whole_block())
                       : line_fft<-1>(smem, smem + ls, 1, ls, a.ph, a.twH);
  col_fwd_store(a, m1, res, threadIdx.x, blockDim.x);
}

// IP: the in-place line DFT, half the shared memory, four CTAs per SM.  The two-buffer
// form runs where columns are short (a few warps per CTA), so registers do not bound its
// occupancy: it gets the registers of two 256-thread CTAs per SM.
template <bool FROM_STATE, int NC, bool IP>
__global__ void __launch_bounds__(kMaxThreads, IP ? 4 : 2) k_col_fwd(IterArgs a) {
  col_fwd_body<FROM_STATE, NC, IP>(a, blockIdx.x);
}

// Two columns per CTA, one per half of the block, each half running its column's in-place
// DFT behind its own named barrier.  A kernel whose CTAs all fit the device at once runs
// every CTA's phases in step, and the dicing (integer work and loads) leaves the FP64 pipe
// idle.  Here both halves first dice column c0; then the first half transforms c0 while
// the second dices c1, and the first half's twiddle-and-store of c0 overlaps the second
// half's DFT of c1.  The FP64 pipe has work while most of the dicing runs.
// Each half has kMaxThreads threads (layouts whose columns take kMaxThreads threads).
template <bool FROM_STATE, int NC>
__global__ void __launch_bounds__(2 * kMaxThreads, 2) k_col_fwd_ws(IterArgs a) {
  extern __shared__ cplx smem[];
  const int ls = a.ls_col;
  constexpr int half = kMaxThreads;
  const int c0 = 2 * (int)blockIdx.x, c1 = c0 + 1;
  const bool second = (int)threadIdx.x >= half;
  const Grp g{(int)threadIdx.x & (half - 1), half, second ? 2 : 1};
  col_fwd_load<FROM_STATE, NC>(a, c0, smem, threadIdx.x, blockDim.x);
  __syncthreads();
  if (second) {
    if (c1 >= a.W) return;  // odd W: the last CTA has one column (its second half waits on nothing)
    col_fwd_load<FROM_STATE, NC>(a, c1, smem + ls, g.tid, half);
    g.sync();
  }
  cplx* buf = second ? smem + ls : smem;
  line_fft_ip<-1>(buf, 1, ls, a.ph, a.twH, g);
  col_fwd_store(a, second ? c1 : c0, buf, g.tid, half);
}

// The row pass's stage values (17.7 KB at W = 576) are copied into shared memory behind
// the four line buffers by one bulk copy, issued before the rows are loaded so the two
// overlap; both DFTs of the pair, forward and inverse, then read them from shared memory.
// L1TW: they are read through L1 instead (no copy, that much less shared memory per CTA).
template <bool R43 = false, bool L1TW = false>
__device__ __forceinline__ void row_sq_body(const IterArgs& a, const int c /* 0 .. H/2 */) {
  extern __shared__ cplx smem[];
  __shared__ alignas(8) uint64_t tw_bar;
  const int W = a.W, H = a.H;
  const int ls = a.ls_row;
  const int ra = c, rb = H - c;
  const bool self = (c == 0) || (2 * c == H);
  const int nl = self ? 1 : 2;
  cplx* buf1 = smem + 2 * ls;
  cplx* tws = smem + 4 * ls;
  if (!L1TW) {
    if (threadIdx.x == 0) mbar_init(&tw_bar);
    __syncthreads();
    if (threadIdx.x == 0) bulk_load(tws, a.twW, (uint32_t)a.twW_n * (uint32_t)sizeof(DevCplx), &tw_bar);
  }
  for (int idx = threadIdx.x; idx < nl * W; idx += blockDim.x) {
    const int l = idx >= W;
    const int k1 = idx - l * W;
    smem[l * ls + pad(k1)] = ldc(a.Z + (size_t)(l ? rb : ra) * W + k1);
  }
  if (L1TW) {
    __syncthreads();
  } else {
    const bool ok = mbar_wait(&tw_bar, 0);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(&a.status->flags, kStatusTimeout);
        mbar_wait(&tw_bar, 0);  // the copy may still land in this CTA's shared memory
      }
      return;
    }
  }
  const auto twc = [&] {
    if constexpr (L1TW) return a.twW;
    else return static_cast<const cplx*>(tws);
  }();
  cplx* sp = line_fft<-1, R43>(smem, buf1, nl, ls, a.pw, twc);
  cplx* other = sp == smem ? buf1 : smem;
  const DevCplx* twp = a.twPair + (size_t)ra * W;
  if (!self) {
    for (int t = threadIdx.x; t < W; t += blockDim.x) {
      const int tp = W - 1 - t;
      cplx vk, vkp;
      pair_square(sp[pad(t)], sp[ls + pad(tp)], ld(twp + t), &vk, &vkp);
      sp[pad(t)] = vk;
      sp[ls + pad(tp)] = vkp;
    }
  } else if (c == 0) {
    // row 0: frequency H*t pairs with H*((W - t) mod W)
    for (int t = threadIdx.x; t <= W / 2; t += blockDim.x) {
      const int tp = (W - t) % W;
      cplx vk, vkp;
      pair_square(sp[pad(t)], sp[pad(tp)], ld(twp + t), &vk, &vkp);
      sp[pad(t)] = vk;
      if (tp != t) sp[pad(tp)] = vkp;
    }
  } else {
    // row H/2: frequency H/2 + H*t pairs with H/2 + H*(W-1-t)
    for (int t = threadIdx.x; t < (W + 1) / 2; t += blockDim.x) {
      const int tp = W - 1 - t;
      cplx vk, vkp;
      pair_square(sp[pad(t)], sp[pad(tp)], ld(twp + t), &vk, &vkp);
      sp[pad(t)] = vk;
      if (tp != t) sp[pad(tp)] = vkp;
    }
  }
  __syncthreads();
  const cplx* res = line_fft<+1, R43>(sp, other, nl, ls, a.pw, twc);
  for (int idx = threadIdx.x; idx < nl * W; idx += blockDim.x) {
    const int l = idx >= W;
    const int m1 = idx - l * W;
    const int row = l ? rb : ra;
    st(a.Z2 + (size_t)m1 * H + row, cmulc(res[l * ls + pad(m1)], ld(a.twK2 + (size_t)row * W + m1)));
  }
}

__global__ void __launch_bounds__(kRowThreads, 3) k_row_sq(IterArgs a) { row_sq_body(a, blockIdx.x); }
// Row plans of radices 4, 3 and 2 only: 64 registers or fewer, so four CTAs of 256 threads
// fit an SM's registers, and with L1TW its shared memory too.
template <bool L1TW>
__global__ void __launch_bounds__(kRowThreads, 4) k_row_sq43(IterArgs a) {
  row_sq_body<true, L1TW>(a, blockIdx.x);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  return v;
}

// bits that product j can place into words j..j+n, natural order (plain form)
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

__device__ __forceinline__ long long round_word(double x, int span, unsigned long long* emax, unsigned* fl) {
  unsigned long long e;
  int big = 0;
  const long long r = round_ll_bits(x, &e, &big);
  *emax = e > *emax ? e : *emax;
  const unsigned long long mag = (unsigned long long)(r < 0 ? -r : r);
  if (big) *fl |= kStatusBig;
  if (span < 63 && (mag >> span) != 0ull) *fl |= kStatusSlice;
  return r;
}

// column m1 of the row pass's output (contiguous in Z2) into buf
__device__ __forceinline__ void col_inv_load(const IterArgs& a, const int m1, cplx* buf, int tid, int nth) {
  const int H = a.H;
  for (int k2 = tid; k2 < H; k2 += nth) buf[pad(k2)] = ldc(a.Z2 + (size_t)m1 * H + k2);
}

// Unweight, round, -2 at word 0, range checks and round-off maximum for column m1 from
// the inverse DFT in res; the inverse weights and spans from shared memory (PF: ai_s,
// sp_s) or from the column-major tables.
template <bool PF>
__device__ __forceinline__ void col_inv_round(const IterArgs& a, const int m1, const cplx* res,
                                              const double* ai_s, const unsigned char* sp_s, int tid, int nth) {
  const int H = a.H;
  unsigned long long emax = 0;
  unsigned fl = 0;
  for (int m2 = tid; m2 < H; m2 += nth) {
    const int s0 = 2 * (m1 * H + m2);
    const cplx v = res[pad(m2)];
    const double2 ai = PF ? make_double2(ai_s[2 * m2], ai_s[2 * m2 + 1])
                          : __ldg(reinterpret_cast<const double2*>(a.Ainv + s0));
    const uchar2 sp = PF ? make_uchar2(sp_s[2 * m2], sp_s[2 * m2 + 1])
                         : __ldg(reinterpret_cast<const uchar2*>(a.span + s0));
    long long r0 = round_word(v.re * ai.x, sp.x, &emax, &fl);
    const long long r1 = round_word(v.im * ai.y, sp.y, &emax, &fl);
    if (s0 == 0) r0 -= 2;  // word 0: the -2 of the LL step, exact on the rounded integer
    *reinterpret_cast<longlong2*>(a.ll + s0) = make_longlong2(r0, r1);
  }
  finish_status(a, emax, fl);
}

// PF (with IP, H a multiple of 8): the column's inverse weights and spans (18 H bytes,
// contiguous in the column-major tables) are brought into shared memory behind the line
// buffer by two bulk copies issued at the start, so the rounding loop after the DFT does
// not wait on global loads.
template <bool IP = false, bool PF = false>
__device__ __forceinline__ void col_inv_body(const IterArgs& a, const int m1) {
  static_assert(!PF || IP, "the prefetch area follows the single in-place line buffer");
  extern __shared__ cplx smem[];
  __shared__ alignas(8) uint64_t pf_bar;
  const int H = a.H;
  const int ls = a.ls_col;
  double* ai_s = reinterpret_cast<double*>(smem + ls);
  unsigned char* sp_s = reinterpret_cast<unsigned char*>(ai_s + 2 * H);
  if (PF) {
    if (threadIdx.x == 0) mbar_init(&pf_bar, 2);
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_load(ai_s, a.Ainv + (size_t)2 * m1 * H, 16u * (uint32_t)H, &pf_bar);
      bulk_load(sp_s, a.span + (size_t)2 * m1 * H, 2u * (uint32_t)H, &pf_bar);
    }
  }
  col_inv_load(a, m1, smem, threadIdx.x, blockDim.x);
  __syncthreads();
  const cplx* res = IP ? line_fft_ip<+1>(smem, 1, ls, a.ph, a.twH, whole_block())
                       : line_fft<+1>(smem, smem + ls, 1, ls, a.ph, a.twH);
  if (PF) {
    const bool ok = mbar_wait(&pf_bar, 0);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(&a.status->flags, kStatusTimeout);
        mbar_wait(&pf_bar, 0);  // the copies may still land in this CTA's shared memory
      }
      return;
    }
  }
  col_inv_round<PF>(a, m1, res, ai_s, sp_s, threadIdx.x, blockDim.x);
}

template <bool IP, bool PF>
__global__ void __launch_bounds__(kMaxThreads, IP && !PF ? 4 : 3) k_col_inv(IterArgs a) {
  col_inv_body<IP, PF>(a, blockIdx.x);
}

// Two columns per CTA as in k_col_fwd_ws: both halves load column c0; the first half's
// inverse DFT of c0 overlaps the second half's load of c1, and the first half's rounding
// and stores of c0 overlap the second half's DFT of c1.
__global__ void __launch_bounds__(2 * kMaxThreads, 2) k_col_inv_ws(IterArgs a) {
  extern __shared__ cplx smem[];
  const int ls = a.ls_col;
  constexpr int half = kMaxThreads;
  const int c0 = 2 * (int)blockIdx.x, c1 = c0 + 1;
  const bool second = (int)threadIdx.x >= half;
  const Grp g{(int)threadIdx.x & (half - 1), half, second ? 2 : 1};
  col_inv_load(a, c0, smem, threadIdx.x, blockDim.x);
  __syncthreads();
  if (second) {
    if (c1 >= a.W) return;
    col_inv_load(a, c1, smem + ls, g.tid, half);
    g.sync();
  }
  cplx* buf = second ? smem + ls : smem;
  line_fft_ip<+1>(buf, 1, ls, a.ph, a.twH, g);
  col_inv_round<false>(a, second ? c1 : c0, buf, nullptr, nullptr, g.tid, half);
}

// ---------------------------------------------------------------------------
// Batched kernels: many tests advance together.  units[blockIdx.x] = (test, local
// unit); each test's arguments come from the descriptor table.  Dynamic shared memory
// and block size are the maxima over the batch; the line FFTs loop over butterflies,
// so a smaller test simply leaves threads idle in some stages.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_desc(const IterArgs* __restrict__ tests, int t, IterArgs& sa) {
  // IterArgs is a plain struct of ints and pointers: copy it word by word
  const int* src = reinterpret_cast<const int*>(tests + t);
  int* dst = reinterpret_cast<int*>(&sa);
  for (int i = threadIdx.x; i < (int)(sizeof(IterArgs) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

template <bool FROM_STATE>
__global__ void __launch_bounds__(kMaxThreads, 2) kb_col_fwd(const IterArgs* __restrict__ tests,
                                                             const int2* __restrict__ units) {
  __shared__ IterArgs sa;
  const int2 u = units[blockIdx.x];
  load_desc(tests, u.x, sa);
  switch (sa.n) {
    case 2: col_fwd_body<FROM_STATE, 2>(sa, u.y); break;
    case 3: col_fwd_body<FROM_STATE, 3>(sa, u.y); break;
    case 4: col_fwd_body<FROM_STATE, 4>(sa, u.y); break;
    case 5: col_fwd_body<FROM_STATE, 5>(sa, u.y); break;
    default: col_fwd_body<FROM_STATE, 6>(sa, u.y); break;
  }
}

// Row pairs c0 .. c0 + k - 1 of one test in one CTA (a batch unit): pair i's rows c and
// H - c are line slots 2i and 2i + 1, and all 2k lines go through each stage together, so
// a short row's stages fill more of the block and the unit's fixed costs (descriptor,
// stage values, barriers) are shared.  A self-paired row (c = 0 or H/2) has slot 2i only;
// its slot 2i + 1 is zero-filled, transformed for nothing and not stored.  Every line's
// arithmetic is row_sq_body's, so the products are the same bit for bit.
__device__ __forceinline__ void row_sq_pairs(const IterArgs& a, const int c0, const int k) {
  extern __shared__ cplx smem[];
  __shared__ alignas(8) uint64_t tw_bar;
  const int W = a.W, H = a.H;
  const int ls = a.ls_row;
  const int nl = 2 * k;
  cplx* buf1 = smem + nl * ls;
  cplx* tws = smem + 2 * nl * ls;
  if (threadIdx.x == 0) mbar_init(&tw_bar);
  __syncthreads();
  if (threadIdx.x == 0) bulk_load(tws, a.twW, (uint32_t)a.twW_n * (uint32_t)sizeof(DevCplx), &tw_bar);
  for (int idx = threadIdx.x; idx < nl * W; idx += blockDim.x) {
    const int l = idx / W;
    const int k1 = idx - l * W;
    const int c = c0 + (l >> 1);
    const bool mirror = l & 1;
    const bool self = c == 0 || 2 * c == H;
    smem[l * ls + pad(k1)] = mirror && self ? mk(0.0, 0.0) : ldc(a.Z + (size_t)(mirror ? H - c : c) * W + k1);
  }
  {
    const bool ok = mbar_wait(&tw_bar, 0);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(&a.status->flags, kStatusTimeout);
        mbar_wait(&tw_bar, 0);  // the copy may still land in this CTA's shared memory
      }
      return;
    }
  }
  const cplx* twc = tws;
  cplx* sp = line_fft<-1>(smem, buf1, nl, ls, a.pw, twc);
  cplx* other = sp == smem ? buf1 : smem;
  for (int t = threadIdx.x; t < k * W; t += blockDim.x) {
    const int i = t / W;
    const int tt = t - i * W;
    const int c = c0 + i;
    cplx* la = sp + 2 * i * ls;
    const DevCplx* twp = a.twPair + (size_t)c * W;
    cplx vk, vkp;
    if (c != 0 && 2 * c != H) {
      const int tp = W - 1 - tt;
      pair_square(la[pad(tt)], la[ls + pad(tp)], ld(twp + tt), &vk, &vkp);
      la[pad(tt)] = vk;
      la[ls + pad(tp)] = vkp;
    } else if (c == 0) {
      // row 0: frequency H*t pairs with H*((W - t) mod W)
      if (tt > W / 2) continue;
      const int tp = (W - tt) % W;
      pair_square(la[pad(tt)], la[pad(tp)], ld(twp + tt), &vk, &vkp);
      la[pad(tt)] = vk;
      if (tp != tt) la[pad(tp)] = vkp;
    } else {
      // row H/2: frequency H/2 + H*t pairs with H/2 + H*(W-1-t)
      if (tt >= (W + 1) / 2) continue;
      const int tp = W - 1 - tt;
      pair_square(la[pad(tt)], la[pad(tp)], ld(twp + tt), &vk, &vkp);
      la[pad(tt)] = vk;
      if (tp != tt) la[pad(tp)] = vkp;
    }
  }
  __syncthreads();
  const cplx* res = line_fft<+1>(sp, other, nl, ls, a.pw, twc);
  for (int idx = threadIdx.x; idx < nl * W; idx += blockDim.x) {
    const int l = idx / W;
    const int m1 = idx - l * W;
    const int c = c0 + (l >> 1);
    const bool mirror = l & 1;
    if (mirror && (c == 0 || 2 * c == H)) continue;
    const int row = mirror ? H - c : c;
    st(a.Z2 + (size_t)m1 * H + row, cmulc(res[l * ls + pad(m1)], ld(a.twK2 + (size_t)row * W + m1)));
  }
}

// units[b] = (test, c0 | k << 20): the row pairs c0 .. c0 + k - 1 of that test (one pair:
// the single-test row body)
__global__ void __launch_bounds__(kRowThreads, 3) kb_row_sq(const IterArgs* __restrict__ tests,
                                                            const int2* __restrict__ units) {
  __shared__ IterArgs sa;
  const int2 u = units[blockIdx.x];
  load_desc(tests, u.x, sa);
  const int c0 = u.y & ((1 << 20) - 1), k = u.y >> 20;
  if (k == 1) row_sq_body(sa, c0);
  else row_sq_pairs(sa, c0, k);
}

__global__ void __launch_bounds__(kMaxThreads, 3) kb_col_inv(const IterArgs* __restrict__ tests,
                                                             const int2* __restrict__ units) {
  __shared__ IterArgs sa;
  const int2 u = units[blockIdx.x];
  load_desc(tests, u.x, sa);
  col_inv_body<false>(sa, u.y);
}

cudaError_t set_batch_smem_limits() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(kb_col_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem))) return e;
  if ((e = cudaFuncSetAttribute(kb_col_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem))) return e;
  if ((e = cudaFuncSetAttribute(kb_col_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem))) return e;
  return cudaFuncSetAttribute(kb_row_sq, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
}

cudaError_t launch_batch_iteration(const BatchLaunch& b, cudaStream_t s, bool from_state) {
  if (from_state) kb_col_fwd<true><<<b.ncol, b.t_col, b.sm_col, s>>>(b.tests, b.col_units);
  else kb_col_fwd<false><<<b.ncol, b.t_col, b.sm_col, s>>>(b.tests, b.col_units);
  kb_row_sq<<<b.nrow, b.t_row, b.sm_row, s>>>(b.tests, b.row_units);
  kb_col_inv<<<b.ncol, b.t_col, b.sm_col, s>>>(b.tests, b.col_units);
  return cudaGetLastError();
}

template <bool FS, bool IP>
static cudaError_t set_col_fwd_smem(int bytes) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_col_fwd<FS, 2, IP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd<FS, 3, IP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd<FS, 4, IP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd<FS, 5, IP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  return cudaFuncSetAttribute(k_col_fwd<FS, 6, IP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <bool FS>
static cudaError_t set_col_fwd_ws_smem(int bytes) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_col_fwd_ws<FS, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd_ws<FS, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd_ws<FS, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  if ((e = cudaFuncSetAttribute(k_col_fwd_ws<FS, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
  return cudaFuncSetAttribute(k_col_fwd_ws<FS, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// The attribute is per kernel and process-wide, shared by every plan: it is raised to the
// layout chooser's bound once (a launch's occupancy follows its own dynamic size).
cudaError_t set_fused_smem_limits(const FusedGeom& g) {
  if (g.sm_col > (size_t)kMaxDynSmem || g.sm_cinv > (size_t)kMaxDynSmem || g.sm_row > (size_t)kMaxDynSmem)
    return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = set_col_fwd_ws_smem<false>(kMaxDynSmem))) return e;
  if ((e = set_col_fwd_ws_smem<true>(kMaxDynSmem))) return e;
  if ((e = cudaFuncSetAttribute(k_col_inv_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem))) return e;
  if ((e = set_col_fwd_smem<false, false>(kMaxDynSmem))) return e;
  if ((e = set_col_fwd_smem<true, false>(kMaxDynSmem))) return e;
  if ((e = set_col_fwd_smem<false, true>(kMaxDynSmem))) return e;
  if ((e = set_col_fwd_smem<true, true>(kMaxDynSmem))) return e;
  if ((e = cudaFuncSetAttribute(k_col_inv<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem)))
    return e;
  if ((e = cudaFuncSetAttribute(k_col_inv<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem)))
    return e;
  if ((e = cudaFuncSetAttribute(k_col_inv<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem)))
    return e;
  if ((e = cudaFuncSetAttribute(k_row_sq43<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem)))
    return e;
  if ((e = cudaFuncSetAttribute(k_row_sq43<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem)))
    return e;
  return cudaFuncSetAttribute(k_row_sq, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
}

template <bool FS, bool IP>
static void launch_col_fwd_ip(const IterArgs& a, const FusedGeom& g, cudaStream_t s) {
  switch (a.n) {
    case 2: k_col_fwd<FS, 2, IP><<<a.W, g.t_col, g.sm_col, s>>>(a); break;
    case 3: k_col_fwd<FS, 3, IP><<<a.W, g.t_col, g.sm_col, s>>>(a); break;
    case 4: k_col_fwd<FS, 4, IP><<<a.W, g.t_col, g.sm_col, s>>>(a); break;
    case 5: k_col_fwd<FS, 5, IP><<<a.W, g.t_col, g.sm_col, s>>>(a); break;
    default: k_col_fwd<FS, 6, IP><<<a.W, g.t_col, g.sm_col, s>>>(a); break;
  }
}

template <bool FS>
static void launch_col_fwd_ws(const IterArgs& a, const FusedGeom& g, cudaStream_t s) {
  const int grid = (a.W + 1) / 2, block = 2 * kMaxThreads;
  switch (a.n) {
    case 2: k_col_fwd_ws<FS, 2><<<grid, block, g.sm_col, s>>>(a); break;
    case 3: k_col_fwd_ws<FS, 3><<<grid, block, g.sm_col, s>>>(a); break;
    case 4: k_col_fwd_ws<FS, 4><<<grid, block, g.sm_col, s>>>(a); break;
    case 5: k_col_fwd_ws<FS, 5><<<grid, block, g.sm_col, s>>>(a); break;
    default: k_col_fwd_ws<FS, 6><<<grid, block, g.sm_col, s>>>(a); break;
  }
}

template <bool FS>
static void launch_col_fwd(const IterArgs& a, const FusedGeom& g, cudaStream_t s) {
  if (g.col_ws) launch_col_fwd_ws<FS>(a, g, s);
  else if (g.col_ip) launch_col_fwd_ip<FS, true>(a, g, s);
  else launch_col_fwd_ip<FS, false>(a, g, s);
}

static void launch_col_inv(const IterArgs& a, const FusedGeom& g, cudaStream_t s) {
  if (g.col_ip && g.col_pf) k_col_inv<true, true><<<a.W, g.t_col, g.sm_cinv, s>>>(a);
  else if (g.col_ws) k_col_inv_ws<<<(a.W + 1) / 2, 2 * kMaxThreads, g.sm_cinv, s>>>(a);
  else if (g.col_ip) k_col_inv<true, false><<<a.W, g.t_col, g.sm_cinv, s>>>(a);
  else k_col_inv<false, false><<<a.W, g.t_col, g.sm_cinv, s>>>(a);
}

static void launch_row(const IterArgs& a, const FusedGeom& g, cudaStream_t s) {
  if (g.row_var == 2) k_row_sq43<true><<<a.H / 2 + 1, g.t_row, g.sm_row, s>>>(a);
  else if (g.row_var == 1) k_row_sq43<false><<<a.H / 2 + 1, g.t_row, g.sm_row, s>>>(a);
  else k_row_sq<<<a.H / 2 + 1, g.t_row, g.sm_row, s>>>(a);
}

cudaError_t launch_fused_iteration(const IterArgs& a, const FusedGeom& g, cudaStream_t s, bool from_state) {
  if (from_state) launch_col_fwd<true>(a, g, s);
  else launch_col_fwd<false>(a, g, s);
  launch_row(a, g, s);
  launch_col_inv(a, g, s);
  return cudaGetLastError();
}

cudaError_t launch_fused_kernel(const IterArgs& a, const FusedGeom& g, cudaStream_t s, int which) {
  if (which == 0) launch_col_fwd<false>(a, g, s);
  else if (which == 1) launch_row(a, g, s);
  else launch_col_inv(a, g, s);
  return cudaGetLastError();
}

// natural <-> column-major copy of an int64 word array
__global__ void k_permute_words(IterArgs a, const long long* __restrict__ src, long long* __restrict__ dst,
                                bool to_colmajor) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.N) return;
  const int c = colmajor(a, j);
  if (to_colmajor) dst[c] = src[j];
  else dst[j] = src[c];
}

cudaError_t launch_permute_words(const IterArgs& a, const long long* src, long long* dst, bool to_colmajor,
                                 cudaStream_t s) {
  k_permute_words<<<(a.N + 255) / 256, 256, 0, s>>>(a, src, dst, to_colmajor);
  return cudaGetLastError();
}

// llintToIrrBal<n> over column-major products (fused form), natural-order output.
// host_digit / host_hi / host_status (device addresses of mapped pinned host memory, or
// null): the carry-save state and the status are also stored there.
__global__ void k_dice_perm(IterArgs a, int* host_digit, signed char* host_hi, Status* host_status) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (host_status && j == 0) *host_status = *a.status;  // final: the passes before have ended
  if (j >= a.N) return;
  const int N = a.N;
  const uint32_t f = a.flags[colmajor(a, j)];
  const long long s = dice_sum(a.LO, a.n, f, [&](int i) {
    const int k = j - i;
    return a.ll[colmajor(a, k < 0 ? k + N : k)];
  });
  int d, h;
  balanced_split(s, a.LO + (int)(f & 1), &d, &h);
  a.digit[j] = d;
  a.hi[j] = (signed char)h;
  if (host_digit) {
    host_digit[j] = d;
    host_hi[j] = (signed char)h;
  }
}

// digit[j] += hi[j-1 mod N] (addPseudoBalanced, IrrBaseBalanced.cu:117-125); the caller
// clears hi afterwards, so (digit, 0) is the same carry-save state
__global__ void k_add_carry(IterArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.N) return;
  a.digit[j] += (int)a.hi[j == 0 ? a.N - 1 : j - 1];
}

// The carry-added words straight from the products: word j is the digit of j's digit sum
// plus the carry of word j-1's (each thread dices both), and the carries are cleared.  One
// pass instead of dicing, adding the carries and clearing them.  CM: the fused form's
// column-major products and flags.  host_words / host_status (device addresses of mapped
// pinned host memory, or null): the words and the status are also stored there, so the
// transfer to the host runs under the dicing instead of as copies after it.
template <bool CM>
__global__ void k_dice_words(IterArgs a, int32_t* host_words, Status* host_status) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = a.N;
  if (host_status && j == 0) *host_status = *a.status;  // final: the passes before have ended
  if (j >= N) return;
  auto pos = [&](int k) {
    if (k < 0) k += N;
    return CM ? colmajor(a, k) : k;
  };
  const uint32_t fj = a.flags[pos(j)], fm = a.flags[pos(j - 1)];
  const long long sj = dice_sum(a.LO, a.n, fj, [&](int i) { return a.ll[pos(j - i)]; });
  const long long sm = dice_sum(a.LO, a.n, fm, [&](int i) { return a.ll[pos(j - 1 - i)]; });
  int dj, hj, dm, hm;
  balanced_split(sj, a.LO + (int)(fj & 1), &dj, &hj);
  balanced_split(sm, a.LO + (int)(fm & 1), &dm, &hm);
  a.digit[j] = dj + hm;
  a.hi[j] = 0;
  if (host_words) host_words[j] = dj + hm;
}

cudaError_t launch_dice_words(const IterArgs& a, bool colmajor_layout, cudaStream_t s, int32_t* host_words,
                              Status* host_status) {
  if (colmajor_layout) k_dice_words<true><<<(a.N + 255) / 256, 256, 0, s>>>(a, host_words, host_status);
  else k_dice_words<false><<<(a.N + 255) / 256, 256, 0, s>>>(a, host_words, host_status);
  return cudaGetLastError();
}

cudaError_t launch_add_carry(const IterArgs& a, cudaStream_t s) {
  k_add_carry<<<(a.N + 255) / 256, 256, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(a.hi, 0, (size_t)a.N, s);
}

cudaError_t launch_dice_perm(const IterArgs& a, cudaStream_t s, int* host_digit, signed char* host_hi,
                             Status* host_status) {
  k_dice_perm<<<(a.N + 255) / 256, 256, 0, s>>>(a, host_digit, host_hi, host_status);
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
__global__ void k_plain_pair_square(DevCplx* Z, const DevCplx* __restrict__ pairC, int M) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > M / 2) return;
  const int kp = k == 0 ? 0 : M - k;
  cplx vk, vkp;
  pair_square(ldc(Z + k), ldc(Z + kp), ld(pairC + k), &vk, &vkp);
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
  k_plain_pair_square<<<(a.M / 2 + 1 + T - 1) / T, T, 0, s>>>(src, a.twPair, a.M);
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

// FP64 issue-rate probe on butterfly code: each thread applies the twiddled radix-8 stage
// butterfly of the line DFTs (ratio form, stored values read from shared memory) to eight
// points held in registers, then scales them by 1/8 to keep them bounded, `iters` times.
// 66 + 16 FP64 instructions per round (62 DFMA + 4 DADD in the butterfly, 16 DMUL).
__global__ void k_probe_butterfly(double* out, long long iters) {
  __shared__ cplx tab[32];
  if (threadIdx.x < 32) {
    const double t = 0.01 * (threadIdx.x & 7);
    tab[threadIdx.x] = mk(0.3 + t, 0.9 - t);
    if ((threadIdx.x & 7) == 1) tab[threadIdx.x].im = bits_dbl(0);  // flags word: no i^f rotations
  }
  __syncthreads();
  cplx v[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = mk(threadIdx.x * 1e-3 + q, q * 0.5);
  const int base = (threadIdx.x & 3) * 8;
  for (long long i = 0; i < iters; ++i) {
    stage_dft<8, -1>(v, true, [&](int k) { return tab[base + k]; });
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = mk(v[q].re * 0.125, v[q].im * 0.125);
  }
  double acc = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) acc += v[q].re + v[q].im;
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

cudaError_t probe_butterfly(int blocks, int threads, long long iters, double* out, cudaStream_t s) {
  k_probe_butterfly<<<blocks, threads, 0, s>>>(out, iters);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Resident form: one cluster holds the test (see ResidentGeom in gl_internal.h).  Per
// iteration: (A) each CTA dices its columns' products (the halo words of the columns
// below come from the owners' shared memory), weights, runs the column DFTs and scatters
// the twiddled columns into the row owners' row lines; cluster barrier; (B) each CTA
// runs its row pairs (DFTs, split + square, inverse DFTs) and scatters the twiddled rows
// into the column owners' column lines; cluster barrier; (C) inverse column DFTs, unweight,
// round, -2, products into shared memory; cluster barrier.  The arithmetic is the fused
// kernels' (same line plans, tables and rounding), so the products are identical.
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;

struct ResidentArgs {
  IterArgs a;
  ResidentGeom g;
  int iters;
};

template <int NC>
__global__ void __launch_bounds__(kResidentThreads, 1) k_resident(const __grid_constant__ ResidentArgs ra) {
  cg::cluster_group cl = cg::this_cluster();
  const IterArgs& a = ra.a;
  const ResidentGeom& g = ra.g;
  extern __shared__ __align__(16) unsigned char rsm[];
  const int rank = (int)cl.block_rank();
  const int C = g.C, cw = g.cw, H = a.H, W = a.W, N = a.N;
  const int lsc = a.ls_col, lsr = a.ls_row;
  const int c0 = rank * cw;
  const int npl = (H / 2 - rank) / C + 1;  // my pairs c = rank + C lp <= H/2 (rank < C <= H/2 + 1)
  cplx* zc = reinterpret_cast<cplx*>(rsm + g.o_zc);
  cplx* zc2 = reinterpret_cast<cplx*>(rsm + g.o_zc2);
  cplx* zr = reinterpret_cast<cplx*>(rsm + g.o_zr);
  cplx* zr2 = reinterpret_cast<cplx*>(rsm + g.o_zr2);
  long long* ll = reinterpret_cast<long long*>(rsm + g.o_ll);
  double* A = reinterpret_cast<double*>(rsm + g.o_A);
  double* Ai = reinterpret_cast<double*>(rsm + g.o_Ai);
  unsigned char* fl = rsm + g.o_fl;
  unsigned char* sp = rsm + g.o_sp;
  cplx* K1 = reinterpret_cast<cplx*>(rsm + g.o_K1);
  cplx* pr = reinterpret_cast<cplx*>(rsm + g.o_pr);
  cplx* K2 = reinterpret_cast<cplx*>(rsm + g.o_K2);
  cplx* twH = reinterpret_cast<cplx*>(rsm + g.o_twH);
  cplx* twW = reinterpret_cast<cplx*>(rsm + g.o_twW);
  const int T = blockDim.x, tid = threadIdx.x;

  // own slices of the state and the tables (column-major per-word arrays: my columns
  // are one contiguous block), whole stage tables
  const int nw = cw * 2 * H;            // my words
  const size_t wbase = (size_t)c0 * 2 * H;
  for (int i = tid; i < nw; i += T) {
    ll[i] = a.ll[wbase + i];
    A[i] = a.A[wbase + i];
    Ai[i] = a.Ainv[wbase + i];
    fl[i] = a.flags[wbase + i];
    sp[i] = a.span[wbase + i];
  }
  for (int i = tid; i < cw * H; i += T) K1[i] = ld(a.twK1 + (size_t)c0 * H + i);
  for (int i = tid; i < npl * W; i += T) {
    const int lp = i / W, t = i - lp * W;
    pr[i] = ld(a.twPair + (size_t)(rank + C * lp) * W + t);
  }
  for (int i = tid; i < 2 * npl * W; i += T) {
    const int s = i / W, m1 = i - s * W;
    const int c = rank + C * (s >> 1);
    const int row = (s & 1) ? (H - c) % H : c;
    K2[i] = ld(a.twK2 + (size_t)row * W + m1);
  }
  for (int i = tid; i < g.twH_n; i += T) twH[i] = ld(a.twH + i);
  for (int i = tid; i < g.twW_n; i += T) twW[i] = ld(a.twW + i);
  cl.sync();

  // word j's owner and local index
  auto where = [&](int j, int* owner) {
    const int m = j >> 1;
    const int m2 = m / W;
    const int m1 = m - m2 * W;
    const int o = m1 / cw;
    *owner = o;
    return 2 * ((m1 - o * cw) * H + m2) + (j & 1);
  };

  for (int it = 0; it < ra.iters; ++it) {
    // (A) dice, weight, column DFTs, twiddle, scatter to the row owners
    for (int idx = tid; idx < cw * H; idx += T) {
      const int lc = idx / H, m2 = idx - lc * H;
      const int m1 = c0 + lc;
      const int j0 = 2 * (m1 + W * m2);
      const int s0 = 2 * idx;  // == 2 (lc H + m2)
      long long P[NC + 3];
      P[0] = ll[s0 + 1];
      P[1] = ll[s0];
#pragma unroll
      for (int k = 2; k < NC + 3; ++k) {
        int j = j0 + 1 - k;
        if (j < 0) j += N;
        int o;
        const int li = where(j, &o);
        P[k] = *cl.map_shared_rank(ll + li, o);
      }
      const int jm = j0 == 0 ? N - 1 : j0 - 1;
      int om;
      const int lm = where(jm, &om);
      const uint32_t f0 = fl[s0], f1 = fl[s0 + 1], fm = *cl.map_shared_rank(fl + lm, om);
      const int LO = a.LO;
      auto dice_at = [&](uint32_t f, int off) {
        const long long mask = (1ll << (LO + (int)(f & 1))) - 1;
        const long long v = P[off];
        long long sum = v < 0 ? -((-v) & mask) : (v & mask);
        int shift = 0;
#pragma unroll
        for (int i = 1; i <= NC; ++i) {
          shift += LO + (int)((f >> i) & 1);
          const long long w = P[off + i];
          sum += shift >= 63 ? 0 : (w < 0 ? -(((-w) >> shift) & mask) : ((w >> shift) & mask));
        }
        return sum;
      };
      const long long sw1 = dice_at(f1, 0), sw0 = dice_at(f0, 1), sm1 = dice_at(fm, 2);
      int dm, hm, d0, h0, d1, h1;
      balanced_split(sm1, LO + (int)(fm & 1), &dm, &hm);
      balanced_split(sw0, LO + (int)(f0 & 1), &d0, &h0);
      balanced_split(sw1, LO + (int)(f1 & 1), &d1, &h1);
      zc[lc * lsc + pad(m2)] = mk(A[s0] * dbl_from_int(d0 + hm), A[s0 + 1] * dbl_from_int(d1 + h0));
    }
    __syncthreads();
    {
      const cplx* res = line_fft<-1>(zc, zc2, cw, lsc, a.ph, (const cplx*)twH);
      for (int idx = tid; idx < cw * H; idx += T) {
        const int lc = idx / H, k2 = idx - lc * H;
        const cplx v = cmul(res[lc * lsc + pad(k2)], K1[idx]);
        const int c = k2 <= H / 2 ? k2 : H - k2;
        const int slot = 2 * (c / C) + (k2 == c ? 0 : 1);
        *cl.map_shared_rank(zr + slot * lsr + pad(c0 + lc), c % C) = v;
      }
    }
    cl.sync();

    // (B) row pairs
    {
      const int nl = 2 * npl;
      cplx* s1 = line_fft<-1>(zr, zr2, nl, lsr, a.pw, (const cplx*)twW);
      cplx* other = s1 == zr ? zr2 : zr;
      for (int idx = tid; idx < npl * W; idx += T) {
        const int lp = idx / W, t = idx - lp * W;
        const int c = rank + C * lp;
        cplx* L0 = s1 + (2 * lp) * lsr;
        cplx* L1 = L0 + lsr;
        const cplx cf = pr[idx];
        cplx vk, vkp;
        if (c != 0 && 2 * c != H) {
          const int tp = W - 1 - t;
          pair_square(L0[pad(t)], L1[pad(tp)], cf, &vk, &vkp);
          L0[pad(t)] = vk;
          L1[pad(tp)] = vkp;
        } else if (c == 0) {
          if (t <= W / 2) {
            const int tp = (W - t) % W;
            pair_square(L0[pad(t)], L0[pad(tp)], cf, &vk, &vkp);
            L0[pad(t)] = vk;
            if (tp != t) L0[pad(tp)] = vkp;
          }
        } else if (t < (W + 1) / 2) {
          const int tp = W - 1 - t;
          pair_square(L0[pad(t)], L0[pad(tp)], cf, &vk, &vkp);
          L0[pad(t)] = vk;
          if (tp != t) L0[pad(tp)] = vkp;
        }
      }
      __syncthreads();
      const cplx* res = line_fft<+1>(s1, other, nl, lsr, a.pw, (const cplx*)twW);
      for (int idx = tid; idx < nl * W; idx += T) {
        const int s = idx / W, m1 = idx - s * W;
        const int c = rank + C * (s >> 1);
        if ((s & 1) && (c == 0 || 2 * c == H)) continue;  // a self-paired row has one line
        const int row = (s & 1) ? H - c : c;
        const cplx v = cmulc(res[s * lsr + pad(m1)], K2[idx]);
        const int o = m1 / cw;
        *cl.map_shared_rank(zc + (m1 - o * cw) * lsc + pad(row), o) = v;
      }
    }
    cl.sync();

    // (C) inverse column DFTs, unweight, round, -2
    {
      const cplx* res = line_fft<+1>(zc, zc2, cw, lsc, a.ph, (const cplx*)twH);
      unsigned long long emax = 0;
      unsigned flg = 0;
      for (int idx = tid; idx < cw * H; idx += T) {
        const int lc = idx / H, m2 = idx - lc * H;
        const int s0 = 2 * idx;
        const cplx v = res[lc * lsc + pad(m2)];
        long long r0 = round_word(v.re * Ai[s0], sp[s0], &emax, &flg);
        const long long r1 = round_word(v.im * Ai[s0 + 1], sp[s0 + 1], &emax, &flg);
        if (rank == 0 && idx == 0) r0 -= 2;  // word 0
        ll[s0] = r0;
        ll[s0 + 1] = r1;
      }
      finish_status(a, emax, flg);
    }
    cl.sync();
  }
  for (int i = tid; i < nw; i += T) a.ll[wbase + i] = ll[i];
}

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <int NC>
static cudaError_t resident_attrs(int smem, int C, cudaLaunchConfig_t* cfg, int* clusters) {
  cudaError_t e = cudaFuncSetAttribute(k_resident<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  if (C > 8 && (e = cudaFuncSetAttribute(k_resident<NC>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) !=
                   cudaSuccess)
    return e;
  return cudaOccupancyMaxActiveClusters(clusters, k_resident<NC>, cfg);
}

static cudaError_t resident_fits(int n, int smem, int C, int* clusters) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kResidentThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  switch (n) {
    case 2: return resident_attrs<2>(smem, C, &cfg, clusters);
    case 3: return resident_attrs<3>(smem, C, &cfg, clusters);
    case 4: return resident_attrs<4>(smem, C, &cfg, clusters);
    case 5: return resident_attrs<5>(smem, C, &cfg, clusters);
    default: return resident_attrs<6>(smem, C, &cfg, clusters);
  }
}

cudaError_t resident_geom(const FusedGeom& fg, int twH_n, int twW_n, int n, ResidentGeom* r) {
  const int H = fg.H, W = fg.W;
  for (int C : {8, 16}) {
    if (W % C || H / 2 + 1 < C) continue;
    ResidentGeom g{};
    g.C = C;
    g.cw = W / C;
    g.npl = (H / 2) / C + 1;
    g.threads = kResidentThreads;
    g.twH_n = twH_n;
    g.twW_n = twW_n;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o = align16(o + bytes);
      return (int)at;
    };
    const size_t colb = (size_t)g.cw * fg.ls_col * 16, rowb = (size_t)2 * g.npl * fg.ls_row * 16;
    const size_t words = (size_t)g.cw * 2 * H;
    g.o_zc = take(colb);
    g.o_zc2 = take(colb);
    g.o_zr = take(rowb);
    g.o_zr2 = take(rowb);
    g.o_ll = take(words * 8);
    g.o_A = take(words * 8);
    g.o_Ai = take(words * 8);
    g.o_fl = take(words);
    g.o_sp = take(words);
    g.o_K1 = take((size_t)g.cw * H * 16);
    g.o_pr = take((size_t)g.npl * W * 16);
    g.o_K2 = take((size_t)2 * g.npl * W * 16);
    g.o_twH = take((size_t)twH_n * 16);
    g.o_twW = take((size_t)twW_n * 16);
    if (o > (size_t)200 * 1024) continue;
    g.smem = (int)o;
    int clusters = 0;
    if (resident_fits(n, g.smem, C, &clusters) != cudaSuccess) {
      cudaGetLastError();  // clear a refused configuration
      continue;
    }
    if (clusters < 1) continue;
    *r = g;
    return cudaSuccess;
  }
  return cudaErrorInvalidConfiguration;
}

template <int NC>
static cudaError_t launch_resident_nc(const ResidentArgs& ra, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ra.g.C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(ra.g.C);
  cfg.blockDim = dim3(ra.g.threads);
  cfg.dynamicSmemBytes = ra.g.smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_resident<NC>, ra);
}

cudaError_t launch_resident(const IterArgs& a, const ResidentGeom& g, int iters, cudaStream_t s) {
  ResidentArgs ra;
  ra.a = a;
  ra.g = g;
  ra.iters = iters;
  switch (a.n) {
    case 2: return launch_resident_nc<2>(ra, s);
    case 3: return launch_resident_nc<3>(ra, s);
    case 4: return launch_resident_nc<4>(ra, s);
    case 5: return launch_resident_nc<5>(ra, s);
    default: return launch_resident_nc<6>(ra, s);
  }
}


// Self-test of the bounded wait: an mbarrier that expects one arrival nobody makes.  The
// wait gives up after `tries` polls, the block records kStatusTimeout exactly as the row
// pass does, and the kernel returns; the context stays usable.
__global__ void k_wait_selftest(Status* st, int tries) {
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar);
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0, tries);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(&st->flags, kStatusTimeout);
}

cudaError_t launch_wait_selftest(Status* st, int tries, cudaStream_t s) {
  k_wait_selftest<<<1, 64, 0, s>>>(st, tries);
  return cudaGetLastError();
}
}  // namespace gl
