// gl_internal.h -- plan layout and kernel launch interface (not part of the C ABI).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gpulucas.h"

namespace gl {

// Line FFTs of the fused form use radices <= kMaxRadix and about kElemsPerThread
// points per thread: a radix-8 butterfly keeps 8 complex values (32 registers) live,
// so 3 CTAs of 256 threads fit an SM's registers.  A twiddled radix-8 stage in ratio form
// costs 2.75 FP64 instructions per point and bit, less than a layered radix-16 one (3).
constexpr int kMaxRadix = 8;
constexpr int kElemsPerThread = 8;
constexpr int kMaxThreads = 256;
constexpr int kRowThreads = 256;
// upper bound of a fused kernel's dynamic shared memory (the layout chooser keeps below)
constexpr int kMaxDynSmem = 112 * 1024;

struct DevCplx {
  double re, im;
};

// Stockham radix sequence of one line DFT of length L (first stage first).
struct LinePlan {
  int L;
  int nst;
  int radix[8];
  int off[8];  // offset of each stage in the stage-ordered twiddle table
};

// Round-off / range status written by the kernels, read by the host between batches.
struct Status {
  unsigned long long maxerr64;  // max |x - rint(x)| * 2^64 over the batch
  unsigned int flags;           // kStatusBig | kStatusSlice
  unsigned int pad;
};
constexpr unsigned kStatusBig = 1u;    // |product| >= 2^51: doubles cannot hold it exactly
constexpr unsigned kStatusSlice = 2u;  // product bits beyond what n+1 slices place
constexpr unsigned kStatusTimeout = 4u; // a bounded device-side wait ran out (kernel returned)

// Geometry of the fused form: the N/2 complex points are an H x W array
// (element m = m1 + W*m2); each column pass CTA takes one column (G = 1), each row
// pass CTA one row pair.  Per-word data of the fused form (products, weights, flags)
// is stored column-major: word j = 2(m1 + W m2) + e lives at 2(m1 H + m2) + e.
struct FusedGeom {
  int W, H, G;
  int col_ip;                // column passes run their DFTs in place (one buffer, 4 CTAs/SM)
  int col_pf;                // with col_ip: the inverse column pass bulk-copies its weights
                             // and spans into shared memory (18 H bytes more)
  int col_ws;                // with col_ip: two columns per CTA, one per half of the block
                             // (2 t_col threads, two in-place line buffers); while one half
                             // transforms its column the other dices or rounds its own (the
                             // inverse pass keeps one column per CTA when col_pf is set)
  int row_var;               // row pass: 0 any radices; 1 radices 4, 3, 2 only (fewer
                             // registers); 2 the same reading its stage values through L1
                             // (no shared-memory copy)
  int rc, rr;                // largest radix of the column / row line plans (8, 4 or 2):
                             // a smaller cap means more, shorter butterflies per stage and
                             // so more threads per line, for lengths too short to fill the GPU
  int ls_col, ls_row;        // padded shared-memory line strides (complex)
  int t_col, t_row;          // threads per CTA
  size_t sm_col, sm_row;     // dynamic shared memory bytes (sm_col: forward column pass)
  size_t sm_cinv;            // inverse column pass (sm_col plus its prefetch area)
  LinePlan pw, ph;
};

struct PlainGeom {
  int nst;
  int radix[40];
  int threads;
};

// Arguments of one iteration (passed by value to every kernel).
struct IterArgs {
  int N, M, W, H, G, LO, n;
  int ls_col, ls_row;
  long long* ll;              // loop-carried products, N int64 (fused: column-major)
  const unsigned char* flags; // bitsPerWord8, N (fused: column-major)
  const unsigned char* span;  // fused: bits product j may place into words j..j+n (column-major)
  const double* A;            // N weights (fused: column-major)
  const double* Ainv;         // N inverse weights with 1/(2N) folded in (fused: column-major)
  DevCplx* Z;                 // M complex work array [H][W]
  DevCplx* Z2;                // M complex: plain, ping-pong; fused, the row pass's output [W][H]
  const DevCplx* twM;         // exp(-2 pi i t/M), t < M
  const DevCplx* twW;         // stage-ordered twiddles of the length-W line DFT
  int twW_n;                  // entries of twW (the row pass copies them to shared memory)
  const DevCplx* twH;         // stage-ordered twiddles of the length-H line DFT
  const DevCplx* twK1;        // w_M^(m1 k2) at m1*H + k2 (column pass output)
  const DevCplx* twPair;      // w_M^(k2 + H k1) at k2*W + k1 (real-signal split)
  const DevCplx* twK2;        // w_M^(m1 k2) at k2*W + m1 (row pass output)
  int* digit;                 // plain: i_signal, N
  signed char* hi;            // plain: i_hiBitArr, N
  Status* status;
  LinePlan pw, ph;
};

// Resident form of a fused plan (short lengths): one thread-block cluster of C CTAs keeps
// the products, the work arrays and every table of the test in distributed shared memory
// and runs many iterations per launch, the three passes separated by cluster barriers.
// CTA r owns columns [r cw, (r+1) cw) and the row pairs c = r, r + C, ... <= H/2.
// Shared-memory regions, byte offsets (all 16-byte aligned):
//   zc, zc2  column lines (cw x ls_col complex, ping-pong)   zr, zr2  row lines (2 npl x ls_row)
//   ll, A, Ai  own columns' products / weights (cw x 2H, 8 B)  fl, sp  flags / span bytes
//   K1  own columns' w^(m1 k2) (cw x H)   pr  own pairs' split coefficients (npl x W)
//   K2  own rows' w^(m1 k2) (2 npl x W)   twH, twW  stage twiddle tables
struct ResidentGeom {
  int C, cw, npl, threads;
  int smem;
  int o_zc, o_zc2, o_zr, o_zr2, o_ll, o_A, o_Ai, o_fl, o_sp, o_K1, o_pr, o_K2, o_twH, o_twW;
  int twH_n, twW_n;
};
constexpr int kResidentThreads = 256;
constexpr int kResidentMaxN = 32768;   // largest N the resident form is tried at (opts.resident = 1)
constexpr int kResidentAutoN = 4096;   // used by default up to here: measured faster than the
                                       // three-launch form (13.8 vs 18.3 us at N = 2048, 16.1 vs
                                       // 19.6 us at 4096; slower from 8192 on)
// smallest cluster first; fills r and returns cudaSuccess if the layout fits one cluster
cudaError_t resident_geom(const FusedGeom& g, int twH_n, int twW_n, int n, ResidentGeom* r);
cudaError_t launch_resident(const IterArgs& a, const ResidentGeom& r, int iters, cudaStream_t s);
cudaError_t launch_wait_selftest(Status* st, int tries, cudaStream_t s);

// A batch of fused-form tests advanced by one set of launches: the descriptor table of
// every test's arguments (device) and the unit maps (test, local column / row pair).
struct BatchLaunch {
  const IterArgs* tests;
  const int2* col_units;
  const int2* row_units;
  int ncol, nrow;
  int t_col, t_row;
  size_t sm_col, sm_row;
};

// launchers (gl_kernels.cu); all asynchronous on `s`
// from_state: the first column pass loads the carry-save state (digit, hi) instead of
// dicing the products, exactly as loadIntToDoubleIBDWT (gpuLucas.cu:730-766) does
cudaError_t launch_fused_iteration(const IterArgs& a, const FusedGeom& g, cudaStream_t s, bool from_state);
// one of the three fused kernels (0 = k_col_fwd, 1 = k_row_sq, 2 = k_col_inv)
cudaError_t launch_fused_kernel(const IterArgs& a, const FusedGeom& g, cudaStream_t s, int which);
cudaError_t launch_plain_iteration(const IterArgs& a, const PlainGeom& g, cudaStream_t s);
cudaError_t launch_set_initial(const IterArgs& a, int mode, cudaStream_t s);
// carry-save state (digit, hi) = dice(ll) for the fused form; plain keeps it already
cudaError_t launch_dice(const IterArgs& a, cudaStream_t s);
// fused form: dice the column-major products into natural-order (digit, hi); host_digit,
// host_hi and host_status, when not null, are device addresses of mapped pinned host
// memory that receive the state and the status as well
cudaError_t launch_dice_perm(const IterArgs& a, cudaStream_t s, int* host_digit = nullptr,
                             signed char* host_hi = nullptr, Status* host_status = nullptr);
// (digit, hi) -> (digit + hi[j-1], 0): the carry-added words, the same state
cudaError_t launch_add_carry(const IterArgs& a, cudaStream_t s);
// products -> (carry-added words, 0) in one pass (colmajor_layout: the fused form's layout);
// host_words / host_status, when not null, are device addresses of mapped pinned host
// memory that receive the words and the status as well
cudaError_t launch_dice_words(const IterArgs& a, bool colmajor_layout, cudaStream_t s,
                              int32_t* host_words = nullptr, Status* host_status = nullptr);
// fused form: natural <-> column-major copies of an int64 word array
cudaError_t launch_permute_words(const IterArgs& a, const long long* src, long long* dst, bool to_colmajor,
                                 cudaStream_t s);
cudaError_t set_fused_smem_limits(const FusedGeom& g);
cudaError_t set_batch_smem_limits();
cudaError_t launch_batch_iteration(const BatchLaunch& b, cudaStream_t s, bool from_state);

// End-of-run normalisation on the device (gl_residue.cu): from the carry-save state
// (digit, hi) the reference's balanced rebalance into `balanced` (N words), then the
// canonical digits' first 64 words, the carries into word 0 and the zero flags into
// `scratch` (residue_scratch_bytes(N) bytes; head at residue_head_offset(N): int32
// head[64], scal[4], flags).  colmajor_flags: the flags table is in the fused layout.
size_t residue_scratch_bytes(int N);
size_t residue_head_offset(int N);
cudaError_t launch_residue(const IterArgs& a, bool colmajor_flags, int32_t* balanced, void* scratch,
                           cudaStream_t s);
cudaError_t probe_fp64(int blocks, int threads, long long iters, double* out, cudaStream_t s);
// 82 FP64 instructions per round and thread (the twiddled radix-8 butterfly and a rescale)
constexpr int kProbeButterflyInstr = 82;
cudaError_t probe_butterfly(int blocks, int threads, long long iters, double* out, cudaStream_t s);

}  // namespace gl
