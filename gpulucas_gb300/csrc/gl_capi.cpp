// gl_capi.cpp -- the C ABI (include/gpulucas.h): plans, iteration, residues and the
// reference-named entry points errorTest / mersenneTest / setSliceAndDice.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gl_internal.h"
#include "gl_plan.h"
#include "gl_tables.h"

using namespace gl;

namespace {

constexpr int kGraphBatch = 64;

int cuda_status(cudaError_t e) { return e == cudaSuccess ? GL_OK : GL_ERR_CUDA; }

#define GL_CUDA(call)                                \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return GL_ERR_CUDA;       \
  } while (0)

template <typename T>
int dev_alloc(gl_plan* pl, T** ptr, size_t count) {
  void* p = nullptr;
  size_t bytes = sizeof(T) * count;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return GL_ERR_NOMEM;
  pl->allocs.push_back(p);
  pl->device_bytes += bytes;
  *ptr = static_cast<T*>(p);
  return GL_OK;
}

bool fill_line_plan(int L, LinePlan* lp, int max_radix = kMaxRadix) {
  std::vector<int> r = radix_plan(L, max_radix);
  if (r.empty() || r.size() > 8) return false;
  lp->L = L;
  lp->nst = (int)r.size();
  for (int i = 0; i < 8; ++i) lp->radix[i] = i < lp->nst ? r[i] : 0;
  return true;
}

int round_up32(int x) { return (x + 31) / 32 * 32; }

// FP64 instructions per point of one stage of radix r of a line DFT.  First stage:
// constant twiddles only (layered DIT, DFT_R).  Later stages: radices 8, 4, 3 in ratio
// form (66, 22, 16 instructions per butterfly), 2 and 16 the layered DIT (3 per point and
// bit), 5 and 7 DFT_R plus one complex product per input.
double stage_ops(int r, bool first) {
  const bool pow2 = (r & (r - 1)) == 0;
  int lg = 0;
  while ((1 << lg) < r) ++lg;
  if (!first && (r == 8 || r == 4 || r == 3)) return (r == 8 ? 66.0 : r == 4 ? 22.0 : 16.0) / r;
  if (pow2) {
    if (!first) return 3.0 * lg;
    return r == 2 ? 2.0 : r == 4 ? 4.0 : r == 8 ? 6.5 : 9.25;  // 16
  }
  const double odd = r == 3 ? 14.0 : r == 5 ? 36.0 : 72.0;  // 7
  return odd / r + (first ? 0.0 : 4.0 * (r - 1) / r);
}

// FP64 instructions per point of one line DFT with the given radices.
double line_ops(const LinePlan& lp) {
  double ops = 0.0;
  for (int s = 0; s < lp.nst; ++s) ops += stage_ops(lp.radix[s], s == 0);
  return ops;
}

// FP64 instructions issued per point of one line DFT when a CTA transforms `nlines` lines
// of the plan together: a stage of radix r has nlines L / r butterflies, one per lane, and
// a warp issues each instruction for all 32 lanes, so the stage costs round_up32(its
// butterflies) / its butterflies times its work.
double line_issue_ops(const LinePlan& lp, int nlines) {
  double ops = 0.0;
  for (int s = 0; s < lp.nst; ++s) {
    const int nb = nlines * lp.L / lp.radix[s];
    ops += stage_ops(lp.radix[s], s == 0) * (double)((nb + 31) / 32 * 32) / nb;
  }
  return ops;
}

// Line plan that issues the fewest FP64 instructions with `nlines` lines per CTA, for
// a batch member (lines short enough that partly filled warps matter): L = 2^a 3^b 5^c 7^d
// with the power of two split into radices 8, 4 and 2 (8 and 4 up to max_radix) in every
// way, and each distinct radix tried as the first stage (the one with constant twiddles);
// the other stages keep the order 8, 4, 2, 3, 5, 7.  At most 8 stages.
bool fill_line_plan_issue(int L, int nlines, int max_radix, LinePlan* lp) {
  if (L < 2) return false;
  int m = L, e[4] = {0, 0, 0, 0};
  const int primes[4] = {2, 3, 5, 7};
  for (int i = 0; i < 4; ++i)
    while (m % primes[i] == 0) {
      m /= primes[i];
      ++e[i];
    }
  if (m != 1) return false;
  double best = 1e300;
  LinePlan out{};
  for (int n8 = 0; 3 * n8 <= e[0]; ++n8) {
    if (n8 && max_radix < 8) break;
    for (int n4 = 0; 3 * n8 + 2 * n4 <= e[0]; ++n4) {
      if (n4 && max_radix < 4) break;
      const int n2 = e[0] - 3 * n8 - 2 * n4;
      const int counts[6] = {n8, n4, n2, e[1], e[2], e[3]};
      const int radices[6] = {8, 4, 2, 3, 5, 7};
      const int nst = n8 + n4 + n2 + e[1] + e[2] + e[3];
      if (nst < 1 || nst > 8) continue;
      for (int f = 0; f < 6; ++f) {
        if (!counts[f]) continue;
        LinePlan c{};
        c.L = L;
        c.nst = nst;
        int k = 0;
        c.radix[k++] = radices[f];
        for (int i = 0; i < 6; ++i)
          for (int j = 0; j < counts[i] - (i == f ? 1 : 0); ++j) c.radix[k++] = radices[i];
        const double cost = line_issue_ops(c, nlines);
        if (cost < best - 1e-9) {
          best = cost;
          out = c;
        }
      }
    }
  }
  if (best >= 1e300) return false;
  *lp = out;
  return true;
}

int padded_stride(int L) { return L + (L >> 4) + 1; }

// FP64-instruction equivalent of one CTA's fixed cost in a batch launch
constexpr double kBatchUnitOverhead = 2000.0;

int stage_offsets(const LinePlan& lp, int* off);

// Shared memory of a row-pass CTA: four line buffers (the pair, ping-pong) and the copy of
// the length-W line DFT's stage values.
size_t row_smem(int W, const LinePlan& pw) {
  int off[8];
  return (size_t)4 * padded_stride(W) * 16 + (size_t)stage_offsets(pw, off) * sizeof(DevCplx);
}

// Radix caps of a layout chosen without timing: below 2^17 complex points a single test
// cannot fill the device with one thread per radix-8 butterfly, and the timed search
// picks radix-4 caps there (more warps per line); a batch member keeps radix 8 (the batch
// fills the device).  Explicit options win.
void model_caps(int M, const gl_plan_opts& o, int sms_override, int* rc, int* rr) {
  const bool small = M < (1 << 17) && !sms_override && !o.fft_h;
  *rc = o.max_radix_col ? o.max_radix_col : (small ? 4 : kMaxRadix);
  *rr = o.max_radix_row ? o.max_radix_row : (small ? 4 : kMaxRadix);
}

// Pick M = W * H for `sms` SMs.  Work units: W columns (column passes, one per CTA)
// and H/2+1 row pairs (row pass).  With equal units per kernel the busiest SM runs
// ceil(units / sms) of them, so the modelled time is the sum over the three kernels
// of ceil(units/sms) * FP64 instructions per unit.  Shared memory per CTA must fit
// twice (two CTAs per SM at least) and blocks stay <= kMaxThreads.
// Every usable column length H of M = W * H with its modelled cost, cheapest first.
std::vector<std::pair<double, int>> ranked_layouts(int M, int sms) {
  if (sms <= 0) sms = 152;
  std::vector<std::pair<double, int>> out;
  for (int H = 2; H <= M / 2; ++H) {
    if (M % H) continue;
    const int W = M / H;
    if (W < 4) continue;  // the forward column pass finds the words below a column with one wrap
    LinePlan a, b;
    // a batch member: line plans and costs by the FP64 instructions issued (a CTA takes
    // one column or one row pair), since its short lines leave warps partly filled
    const bool member = sms == 1;
    if (member ? !fill_line_plan_issue(W, 2, kMaxRadix, &a) || !fill_line_plan_issue(H, 1, kMaxRadix, &b)
               : !fill_line_plan(W, &a) || !fill_line_plan(H, &b))
      continue;
    const size_t smc = (size_t)2 * padded_stride(H) * 16, smr = row_smem(W, a);
    if (smc > (size_t)kMaxDynSmem || smr > (size_t)kMaxDynSmem) continue;
    if ((H + kElemsPerThread - 1) / kElemsPerThread > 4 * kMaxThreads) continue;
    const double col_ops = member ? line_issue_ops(b, 1) : line_ops(b);
    const double row_ops = member ? line_issue_ops(a, 2) : line_ops(a);
    double col = std::ceil((double)W / sms) * H * (col_ops + 6.0);
    double row = std::ceil((double)(H / 2 + 1) / sms) * 2.0 * W * (2.0 * row_ops + 16.0);
    if (member) {
      // its units share the device with the batch's other units, so the fixed cost of a
      // CTA (launch, descriptor copy, barriers, global round trips) is charged per unit,
      // which keeps the lines long enough to amortise it
      col += (double)W * kBatchUnitOverhead;
      row += (double)(H / 2 + 1) * kBatchUnitOverhead;
    }
    double cost = 2.0 * col + row;
    // prefer smaller shared-memory footprints (more resident CTAs) on ties
    cost *= 1.0 + 0.02 * (double)(smc + smr) / (64.0 * 1024);
    out.emplace_back(cost, H);
  }
  std::sort(out.begin(), out.end());
  return out;
}

// Block size of the row pass (two lines of W points): from t0 (one thread per butterfly of
// the largest-radix stage) up to kRowThreads, the smallest multiple of 32 that minimises
// the stages' rounds of butterflies weighted by radix, so that a stage with more, smaller
// butterflies (radix 3 after radix 8) does not leave most warps waiting at its barrier
// while a few run one more round.  W = 576 (8, 8, 3, 3): 160 -> 192 threads.
int row_threads(int W, const LinePlan& pw, int t0) {
  int best = t0;
  long best_cost = -1;
  for (int t = t0; t <= kRowThreads; t += 32) {
    long cost = 0;
    for (int s = 0; s < pw.nst; ++s) {
      const int R = pw.radix[s];
      const int nb = 2 * W / R;
      cost += (long)((nb + t - 1) / t) * R;
    }
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = t;
    }
  }
  return best;
}

// Layout for M: column length `force_h` (0: the model's best) with line plans whose
// largest radix is rc (columns) / rr (rows); each column gets one thread per butterfly
// of its largest-radix stage, each row pair row_threads().
int choose_fused_geom(int M, int force_h, int sms, FusedGeom* g, int rc = kMaxRadix, int rr = kMaxRadix,
                      bool ip = false, bool pf = false, bool ws = false, int row = 0) {
  if ((rc != 8 && rc != 4 && rc != 2) || (rr != 8 && rr != 4 && rr != 2)) return GL_ERR_ARG;
  int bestH = 0;
  for (const auto& c : ranked_layouts(M, sms))
    if (!force_h || c.second == force_h) {
      bestH = c.second;
      break;
    }
  if (!bestH) return GL_ERR_SIZE;
  g->H = bestH;
  g->W = M / bestH;
  g->G = 1;
  g->rc = rc;
  g->rr = rr;
  if (sms == 1) {  // a batch member: the plans that issue the fewest FP64 instructions
    if (!fill_line_plan_issue(g->W, 2, rr, &g->pw) || !fill_line_plan_issue(g->H, 1, rc, &g->ph)) return GL_ERR_SIZE;
  } else if (!fill_line_plan(g->W, &g->pw, rr) || !fill_line_plan(g->H, &g->ph, rc)) {
    return GL_ERR_SIZE;
  }
  g->ls_col = padded_stride(g->H);
  g->ls_row = padded_stride(g->W);
  g->sm_col = (size_t)2 * g->ls_col * 16;
  g->sm_cinv = g->sm_col;
  g->sm_row = row_smem(g->W, g->pw);
  auto threads = [](int points, int per_thread, int cap) {
    int t = round_up32((points + per_thread - 1) / per_thread);
    return t < 64 ? 64 : (t > cap ? cap : t);
  };
  g->t_col = threads(g->H, rc, kMaxThreads);
  g->t_row = row_threads(g->W, g->pw, threads(2 * g->W, rr, kRowThreads));
  g->row_var = 0;
  if (row < 0 || row > 2) return GL_ERR_ARG;
  if (row > 0) {
    for (int s = 0; s < g->pw.nst; ++s) {
      const int R = g->pw.radix[s];
      if (R != 2 && R != 3 && R != 4) return GL_ERR_SIZE;
    }
    g->row_var = row;
    if (row == 2) g->sm_row = (size_t)4 * g->ls_row * 16;  // stage values read through L1
  }
  g->col_ip = 0;
  g->col_pf = 0;
  g->col_ws = 0;
  if (ip || ws) {
    // in place: every column stage has at most (8 / R for radix R = 2^k, 1 for odd R)
    // butterflies per thread, held in registers across the stage's first barrier
    for (int s = 0; s < g->ph.nst; ++s) {
      const int R = g->ph.radix[s];
      const int per = (R & (R - 1)) == 0 ? 8 / R : 1;
      if (g->H / R > per * g->t_col) return GL_ERR_SIZE;
    }
    g->col_ip = 1;
    g->sm_col = g->sm_cinv = (size_t)g->ls_col * 16;
    if (ws) {
      // two columns per CTA: two in-place line buffers; the inverse pass too, unless it
      // prefetches its weights (then it keeps one column per CTA)
      if (g->W < 2 || g->t_col != kMaxThreads) return GL_ERR_SIZE;
      g->col_ws = 1;
      g->sm_col = g->sm_cinv = (size_t)2 * g->ls_col * 16;
      if (g->sm_col > (size_t)kMaxDynSmem) return GL_ERR_SIZE;
    }
    if (pf) {
      if (g->H % 8) return GL_ERR_SIZE;  // bulk copies of 2H bytes must be 16-byte multiples
      g->col_pf = 1;
      g->sm_cinv = (size_t)g->ls_col * 16 + (size_t)18 * g->H;
    }
  }
  return GL_OK;
}

int choose_plain_geom(int M, PlainGeom* g) {
  const int nst = radix_plan_into(M, 4, g->radix, 40);
  if (nst <= 0) return GL_ERR_SIZE;
  g->nst = nst;
  g->threads = 256;
  return GL_OK;
}

// offsets of each stage in a stage-ordered twiddle table (gl_tables.cpp layout) and
// the table length, without computing the values
int stage_offsets(const LinePlan& lp, int* off) {
  int size = 1, Ns = 1;
  for (int s = 0; s < lp.nst; ++s) {
    off[s] = size;
    if (Ns > 1) size += stage_values(lp.radix[s]) * Ns;
    Ns *= lp.radix[s];
  }
  return size;
}

// Device time of one fused iteration with column length H, measured on zero-filled
// buffers (the kernels' time does not depend on the values).  Returns ms, or -1.
double time_layout(int M, int H, int rc, int rr, bool ip, bool pf, bool ws, int row, int n, int sms, int iters,
                   cudaStream_t s) {
  FusedGeom g{};
  if (choose_fused_geom(M, H, sms, &g, rc, rr, ip, pf, ws, row) != GL_OK) return -1.0;
  const int N = 2 * M;
  const int szw = stage_offsets(g.pw, g.pw.off), szh = stage_offsets(g.ph, g.ph.off);
  const size_t bytes[] = {sizeof(long long) * N, (size_t)N, (size_t)N, sizeof(double) * N, sizeof(double) * N,
                          16 * (size_t)M, 16 * (size_t)M, 16 * (size_t)M, 16 * (size_t)M,
                          16 * (size_t)szw, 16 * (size_t)szh, sizeof(int) * N, (size_t)N, sizeof(Status),
                          16 * (size_t)M};
  constexpr int nb = sizeof(bytes) / sizeof(bytes[0]);
  void* buf[nb] = {};
  double ms = -1.0;
  bool ok = true;
  for (int i = 0; i < nb && ok; ++i) ok = cudaMalloc(&buf[i], bytes[i]) == cudaSuccess &&
                                         cudaMemsetAsync(buf[i], 0, bytes[i], s) == cudaSuccess;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ok) ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  if (ok) ok = set_fused_smem_limits(g) == cudaSuccess;
  if (ok) {
    IterArgs a{};
    a.N = N; a.M = M; a.W = g.W; a.H = g.H; a.G = 1; a.LO = 18; a.n = n;
    a.ls_col = g.ls_col; a.ls_row = g.ls_row; a.pw = g.pw; a.ph = g.ph;
    a.ll = (long long*)buf[0]; a.flags = (const unsigned char*)buf[1]; a.span = (const unsigned char*)buf[2];
    a.A = (const double*)buf[3]; a.Ainv = (const double*)buf[4]; a.Z = (DevCplx*)buf[5];
    a.twK1 = (const DevCplx*)buf[6]; a.twPair = (const DevCplx*)buf[7]; a.twK2 = (const DevCplx*)buf[8];
    a.twW = (const DevCplx*)buf[9]; a.twH = (const DevCplx*)buf[10]; a.twW_n = szw;
    a.digit = (int*)buf[11]; a.hi = (signed char*)buf[12]; a.status = (Status*)buf[13];
    a.Z2 = (DevCplx*)buf[14];
    for (int i = 0; i < 2 && ok; ++i) ok = launch_fused_iteration(a, g, s, false) == cudaSuccess;
    ok = ok && cudaEventRecord(e0, s) == cudaSuccess;
    for (int i = 0; i < iters && ok; ++i) ok = launch_fused_iteration(a, g, s, false) == cudaSuccess;
    ok = ok && cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
    float t = 0.f;
    if (ok && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess) ms = t / iters;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(s);
  for (void* b : buf)
    if (b) cudaFree(b);
  return ms;
}

// Autotuned layout for M on this device: the cheapest few column lengths of the cost
// model are timed and the fastest kept, once per (M, SM count) per process.  Below
// 2^17 complex points the lines are too short to fill the GPU with one thread per
// radix-8 butterfly, so the three best lengths are also timed with radix-4 and radix-2
// caps.  The column-pass variants (two buffers, in place, in place with prefetched
// weights, two columns per CTA) are timed on the best lengths, and the winner once more
// with radix-4 rows: a radix-8 row stage of W/8 butterflies per line leaves part of a warp
// idle when 2W/8 is not a multiple of 32 (W = 576: 144 butterflies on 192 threads), while
// radix-4 stages fill whole warps.
struct TunedLayout {
  int H = 0, rc = kMaxRadix, rr = kMaxRadix, row = 0;
  bool ip = false, pf = false, ws = false;
  double ms = 0.0;
};
std::mutex g_tune_mutex;
std::map<std::pair<int, int>, TunedLayout> g_tune_cache;

TunedLayout autotune_layout(int M, int n, int sms, cudaStream_t s, double* ms_out) {
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find({M, sms});
    if (it != g_tune_cache.end()) {
      if (ms_out) *ms_out = it->second.ms;
      return it->second;
    }
  }
  const auto ranked = ranked_layouts(M, sms);
  TunedLayout best;
  double best_ms = 1e300;
  const int iters = M >= (1 << 18) ? 10 : 40;
  auto consider = [&](int H, int rc, int rr, bool ip, bool pf = false, bool ws = false, int row = 0) {
    const double ms = time_layout(M, H, rc, rr, ip, pf, ws, row, n, sms, iters, s);
    if (ms > 0.0 && ms < best_ms) {
      best_ms = ms;
      best.H = H;
      best.rc = rc;
      best.rr = rr;
      best.ip = ip;
      best.pf = pf;
      best.ws = ws;
      best.row = row;
    }
  };
  for (size_t i = 0; i < ranked.size() && i < 6; ++i) {
    consider(ranked[i].second, kMaxRadix, kMaxRadix, false);
    // the in-place column passes (half the shared memory, 4 CTAs per SM); long columns
    // also with prefetched weights and two per CTA
    consider(ranked[i].second, kMaxRadix, kMaxRadix, true);
    if (M >= (1 << 17)) {
      consider(ranked[i].second, kMaxRadix, kMaxRadix, true, true);
      consider(ranked[i].second, kMaxRadix, kMaxRadix, true, false, true);
      consider(ranked[i].second, kMaxRadix, kMaxRadix, true, true, true);
    }
  }
  if (M >= (1 << 17) && best.H) {
    const TunedLayout b = best;
    consider(b.H, b.rc, 4, b.ip, b.pf, b.ws);
  }
  if (best.H) {
    // the row pass compiled for radices 4, 3, 2 only, with its stage values in shared
    // memory or read through L1 (where the row plan allows it; otherwise not timed)
    const TunedLayout b = best;
    consider(b.H, b.rc, b.rr, b.ip, b.pf, b.ws, 1);
    consider(b.H, b.rc, b.rr, b.ip, b.pf, b.ws, 2);
  }
  if (M < (1 << 17))
    for (size_t i = 0; i < ranked.size() && i < 3; ++i) {
      consider(ranked[i].second, 4, kMaxRadix, false);
      consider(ranked[i].second, kMaxRadix, 4, false);
      consider(ranked[i].second, 4, 4, false);
      consider(ranked[i].second, 4, 4, true);
      consider(ranked[i].second, 4, kMaxRadix, true);
      // radix-2 stages: a little more FP64 work per point and bit (3 against 2.75 for
      // radix 4 in ratio form), twice the butterflies per stage, so twice the warps to hide
      // FP64 latency on short lines
      consider(ranked[i].second, 2, 4, false);
      consider(ranked[i].second, 4, 2, false);
      consider(ranked[i].second, 2, 2, false);
    }
  if (!best.H) return best;
  best.ms = best_ms;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune_cache[{M, sms}] = best;
  if (ms_out) *ms_out = best_ms;
  return best;
}

void free_plan(gl_plan* pl) {
  if (!pl) return;
  if (pl->device >= 0) cudaSetDevice(pl->device);
  if (pl->gexec) cudaGraphExecDestroy(pl->gexec);
  if (pl->hw_exec) cudaGraphExecDestroy(pl->hw_exec);
  for (void* p : pl->allocs) cudaFree(p);
  if (pl->h_status) cudaFreeHost(pl->h_status);
  if (pl->h_res) cudaFreeHost(pl->h_res);
  if (pl->ev0) cudaEventDestroy(pl->ev0);
  if (pl->ev1) cudaEventDestroy(pl->ev1);
  if (pl->stream) cudaStreamDestroy(pl->stream);
  delete pl;
}

int launch_iterations(gl_plan* pl, int64_t k) {
  for (int64_t i = 0; i < k; ++i) {
    cudaError_t e;
    if (pl->mode == GL_MODE_PLAIN) {
      e = launch_plain_iteration(pl->args, pl->pg, pl->stream);
    } else {
      e = launch_fused_iteration(pl->args, pl->fg, pl->stream, pl->from_state);
      pl->from_state = false;
    }
    if (e != cudaSuccess) return GL_ERR_CUDA;
  }
  return GL_OK;
}

// Enqueue k iterations, with batches of kGraphBatch replayed from one CUDA graph.
int enqueue(gl_plan* pl, int64_t k) {
  if (k <= 0) return GL_OK;
  int rc;
  if (pl->from_state) {  // the state-loading first pass is never captured
    if ((rc = launch_iterations(pl, 1)) != GL_OK) return rc;
    --k;
  }
  if (pl->resident) {  // one cluster launch runs them all
    while (k > 0) {
      const int chunk = (int)std::min<int64_t>(k, 1 << 30);
      GL_CUDA(launch_resident(pl->args, pl->rg, chunk, pl->stream));
      k -= chunk;
    }
    return GL_OK;
  }
  if (pl->use_graphs && k >= kGraphBatch) {
    if (!pl->gexec) {
      cudaGraph_t graph = nullptr;
      GL_CUDA(cudaStreamBeginCapture(pl->stream, cudaStreamCaptureModeThreadLocal));
      int lrc = launch_iterations(pl, kGraphBatch);
      cudaError_t ec = cudaStreamEndCapture(pl->stream, &graph);
      if (lrc != GL_OK || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return GL_ERR_CUDA;
      }
      cudaError_t ei = cudaGraphInstantiate(&pl->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess) {
        pl->gexec = nullptr;
        return GL_ERR_CUDA;
      }
      pl->gexec_iters = kGraphBatch;
    }
    while (k >= pl->gexec_iters) {
      GL_CUDA(cudaGraphLaunch(pl->gexec, pl->stream));
      k -= pl->gexec_iters;
    }
  }
  return launch_iterations(pl, k);
}

// Wait for the stream and fold the device status into the plan.
int read_status(gl_plan* pl, double* maxerr_out) {
  GL_CUDA(cudaMemcpyAsync(pl->h_status, pl->args.status, sizeof(Status), cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  const double e = std::ldexp((double)pl->h_status->maxerr64, -64);
  if (e > pl->run_maxerr) pl->run_maxerr = e;
  if (maxerr_out) *maxerr_out = e;
  if (pl->h_status->flags & kStatusTimeout) return GL_ERR_TIMEOUT;
  if (pl->h_status->flags) return GL_ERR_OVERFLOW;
  if (e >= pl->error_limit) return GL_ERR_ROUNDOFF;
  return GL_OK;
}

}  // namespace

extern "C" {

int gl_version(void) { return 100; }

const char* gl_error_string(int s) {
  switch (s) {
    case GL_OK: return "ok";
    case GL_ERR_ARG: return "bad argument";
    case GL_ERR_RATIO: return "p/N outside the carry-depth table (ratio >= 22)";
    case GL_ERR_SIZE: return "N must be even with N/2 = 2^a 3^b 5^c 7^d and a usable FFT layout";
    case GL_ERR_CUDA: return "CUDA runtime error";
    case GL_ERR_NOMEM: return "out of memory";
    case GL_ERR_ROUNDOFF: return "round-off error reached the limit";
    case GL_ERR_OVERFLOW: return "product out of the exactly representable / sliced range";
    case GL_ERR_NODEVICE: return "no CUDA device";
    case GL_ERR_IO: return "checkpoint I/O error";
    case GL_ERR_CHECKPOINT: return "checkpoint does not match the test";
    case GL_ERR_STATE: return "call not valid in this state";
    case GL_ERR_TOO_LARGE: return "N exceeds 65536, the limit of gl_iterate_noalloc";
    case GL_ERR_TIMEOUT: return "a bounded device-side wait ran out";
    default: return "unknown status";
  }
}

int gl_default_opts(gl_plan_opts* o) {
  if (!o) return GL_ERR_ARG;
  std::memset(o, 0, sizeof(*o));
  o->mode = GL_MODE_FUSED;
  o->device = 0;
  o->error_limit = 0.4;
  o->check_every = 1000;
  o->use_graphs = 1;
  o->autotune = 1;
  return GL_OK;
}

int setSliceAndDice(int testPrime, int signalSize) {
  if (testPrime <= 2 || signalSize <= 0) return GL_ERR_ARG;
  int n = slice_depth(testPrime, signalSize);
  return n < 0 ? GL_ERR_RATIO : n;
}

int gl_plan_create(int p, int N, const gl_plan_opts* opts, gl_plan** out) {
  return gl_plan_create_ex(p, N, opts, opts && opts->batch_layout ? 1 : 0, out);
}

}  // extern "C"

cudaError_t gl_make_stream(cudaStream_t* s, int level) {
  int least = 0, greatest = 0;
  if (level) {
    const cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
  }
  const int prio = level == 1 ? greatest : (level == 2 ? (greatest + least) / 2 : least);
  return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, prio);
}

void gl_plan_note_external_iterations(gl_plan* pl, int64_t iters) {
  pl->iters_done += iters;
  pl->from_state = false;
  pl->carry_valid = pl->mode == GL_MODE_PLAIN;
}

double gl_model_iteration_cost(int M, int sms) {
  const auto r = ranked_layouts(M, sms);
  return r.empty() ? HUGE_VAL : r.front().first;
}

double gl_plan_unit_cost(const gl_plan* pl, bool row) {
  if (row) return 2.0 * pl->fg.W * (2.0 * line_ops(pl->fg.pw) + 16.0);
  return pl->fg.H * (line_ops(pl->fg.ph) + 6.0);
}

int gl_plan_create_ex(int p, int N, const gl_plan_opts* opts, int sms_override, gl_plan** out) {
  if (!out) return GL_ERR_ARG;
  *out = nullptr;
  gl_plan_opts o;
  if (opts) o = *opts;
  else gl_default_opts(&o);
  if (N == 0 && p >= 3) {
    int rc0 = gl_find_signal_size(p, &o, &N, nullptr, nullptr);
    if (rc0 != GL_OK) return rc0;
  }
  if (p < 3 || N < 16 || (N & 1) || N > p) return GL_ERR_ARG;
  if (o.mode != GL_MODE_FUSED && o.mode != GL_MODE_PLAIN) return GL_ERR_ARG;
  if (!(o.error_limit > 0.0 && o.error_limit <= 0.5) || o.check_every < 1) return GL_ERR_ARG;
  if (o.high_priority < 0 || o.high_priority > 2) return GL_ERR_ARG;
  const int n = slice_depth(p, N);
  if (n < 0) return GL_ERR_RATIO;
  const int M = N / 2;
  FusedGeom fg{};
  PlainGeom pg{};
  if (o.cols_per_cta > 1) return GL_ERR_ARG;  // the column passes take one column per CTA
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GL_ERR_NODEVICE;
  if (o.device < 0 || o.device >= ndev) return GL_ERR_ARG;
  if (cudaSetDevice(o.device) != cudaSuccess) return GL_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o.device) != cudaSuccess) return GL_ERR_CUDA;
  if (sms_override > 0) sms = sms_override;
  int force_h = o.fft_h, cap_c = kMaxRadix, cap_r = kMaxRadix;
  model_caps(M, o, sms_override, &cap_c, &cap_r);
  // Short lengths: the resident form (one cluster, the whole test in shared memory) when
  // a layout with W divisible by the cluster size fits; it replaces the layout search.
  bool resident = false;
  ResidentGeom rg{};
  if (o.mode == GL_MODE_FUSED && !sms_override && !force_h &&
      (o.resident > 0 ? N <= kResidentMaxN : (o.resident == 0 && N <= kResidentAutoN))) {
    // radix 4: each CTA's lines are short, and more, shorter butterflies keep more warps
    // issuing FP64 work (measured: 13.8 us at N = 2048 against 16.6 us with radix 8)
    const int rcap = o.max_radix_col ? o.max_radix_col : 4, wcap = o.max_radix_row ? o.max_radix_row : 4;
    for (const auto& c : ranked_layouts(M, sms)) {
      FusedGeom t{};
      if (choose_fused_geom(M, c.second, sms, &t, rcap, wcap) != GL_OK) continue;
      int offh[8], offw[8];
      const int nh = stage_offsets(t.ph, offh), nw = stage_offsets(t.pw, offw);
      if (resident_geom(t, nh, nw, n, &rg) == cudaSuccess) {
        resident = true;
        force_h = c.second;
        cap_c = rcap;
        cap_r = wcap;
        break;
      }
    }
    cudaGetLastError();
  }
  if (o.resident > 0 && !resident) return GL_ERR_SIZE;
  bool col_ip = false, col_pf = false, col_ws = false;
  int row_var = 0;
  if (o.mode == GL_MODE_FUSED && !force_h && o.autotune && !sms_override) {
    const TunedLayout t = autotune_layout(M, n, sms, 0, nullptr);
    if (t.H) {
      force_h = t.H;
      if (!o.max_radix_col) cap_c = t.rc;
      if (!o.max_radix_row) cap_r = t.rr;
      col_ip = t.ip && !resident;
      col_pf = col_ip && t.pf;
      col_ws = col_ip && t.ws;
      row_var = resident ? 0 : t.row;
    }
  }
  if (o.row_pass) {
    if (o.row_pass < -1 || o.row_pass > 2) return GL_ERR_ARG;
    row_var = o.row_pass > 0 && !resident ? o.row_pass : 0;
  }
  if (o.col_inplace) {
    if (o.col_inplace > 4) return GL_ERR_ARG;
    col_ip = o.col_inplace > 0 && !resident && !sms_override;
    col_pf = col_ip && (o.col_inplace == 2 || o.col_inplace == 4);
    col_ws = col_ip && (o.col_inplace == 3 || o.col_inplace == 4);
  }
  int rc = o.mode == GL_MODE_FUSED
               ? choose_fused_geom(M, force_h, sms, &fg, cap_c, cap_r, col_ip, col_pf, col_ws, row_var)
               : choose_plain_geom(M, &pg);
  if (rc == GL_ERR_SIZE && col_ip && o.col_inplace <= 0)  // the searched layout cannot: two buffers
    rc = choose_fused_geom(M, force_h, sms, &fg, cap_c, cap_r, false);
  if (rc != GL_OK) return rc;

  gl_plan* pl = new (std::nothrow) gl_plan();
  if (!pl) return GL_ERR_NOMEM;
  pl->p = p; pl->N = N; pl->M = M; pl->LO = p / N; pl->n = n;
  pl->mode = o.mode; pl->device = o.device;
  pl->error_limit = o.error_limit; pl->check_every = o.check_every; pl->use_graphs = o.use_graphs;
  pl->fg = fg; pl->pg = pg;

#define GL_TRY(x)             \
  do {                        \
    int r_ = (x);             \
    if (r_ != GL_OK) {        \
      free_plan(pl);          \
      return r_;              \
    }                         \
  } while (0)
#define GL_TRYC(x) GL_TRY(cuda_status(x))

  GL_TRYC(gl_make_stream(&pl->stream, o.high_priority));
  GL_TRYC(cudaEventCreate(&pl->ev0));
  GL_TRYC(cudaEventCreate(&pl->ev1));
  GL_TRYC(cudaMallocHost((void**)&pl->h_status, sizeof(Status)));

  std::vector<int32_t> bits;
  std::vector<uint8_t> flags;
  std::vector<double> A, Ainv;
  std::vector<HostCplx> twM;
  word_tables(p, N, bits, flags);
  // the row pass produces V = DFT_M(z_even + i z_odd) exactly, so the unnormalized
  // inverse returns M z: Ainv = 1/(M A) (the reference's (1/A)/N with N = 2M)
  weight_tables(p, N, (double)M, A, Ainv);
  twiddle_table(M, twM);

  IterArgs& a = pl->args;
  a.N = N; a.M = M; a.LO = pl->LO; a.n = n;
  long long* ll;
  unsigned char *fl, *span = nullptr;
  double *dA, *dAi;
  DevCplx *Z, *Z2 = nullptr, *dtwM = nullptr, *dtwW = nullptr, *dtwH = nullptr;
  DevCplx *dK1 = nullptr, *dPair = nullptr, *dK2 = nullptr;
  int* digit;
  signed char* hi;
  Status* status;
  GL_TRY(dev_alloc(pl, &ll, N));
  GL_TRY(dev_alloc(pl, &fl, N));
  GL_TRY(dev_alloc(pl, &dA, N));
  GL_TRY(dev_alloc(pl, &dAi, N));
  GL_TRY(dev_alloc(pl, &Z, M));
  GL_TRY(dev_alloc(pl, &digit, N));
  GL_TRY(dev_alloc(pl, &hi, N));
  GL_TRY(dev_alloc(pl, &status, 1));
  GL_TRY(dev_alloc(pl, &pl->rscratch, residue_scratch_bytes(N)));
  GL_TRYC(cudaMallocHost((void**)&pl->h_res, sizeof(int32_t) * 72));
  if (o.mode == GL_MODE_PLAIN) {
    std::vector<HostCplx> pc((size_t)M);
    parallel_for(M, [&](int64_t b, int64_t e) {
      for (int64_t k = b; k < e; ++k) pc[k] = pair_coeff(k, M);
    });
    GL_TRY(dev_alloc(pl, &Z2, M));
    GL_TRY(dev_alloc(pl, &dtwM, M));
    GL_TRY(dev_alloc(pl, &dPair, M));
    GL_TRYC(cudaMemcpyAsync(dtwM, twM.data(), sizeof(DevCplx) * M, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dPair, pc.data(), sizeof(DevCplx) * M, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(fl, flags.data(), N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dA, A.data(), sizeof(double) * N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dAi, Ainv.data(), sizeof(double) * N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaStreamSynchronize(pl->stream));  // host tables go out of scope
  } else {
    const int W = fg.W, H = fg.H;
    // per-word tables in column-major order: word j = 2(m1 + W m2) + e -> 2(m1 H + m2) + e
    std::vector<uint8_t> fl_c(N), span_c(N);
    std::vector<double> A_c(N), Ai_c(N);
    for (int j = 0; j < N; ++j) {
      const int m = j >> 1, m1 = m % W, m2 = m / W;
      const int c = 2 * (m1 * H + m2) + (j & 1);
      fl_c[c] = flags[j];
      A_c[c] = A[j];
      Ai_c[c] = Ainv[j];
      int tot = 0;
      for (int i = 0; i <= n; ++i) tot += bits[(j + i) % N];
      span_c[c] = (uint8_t)(tot > 255 ? 255 : tot);
    }
    std::vector<int> rw(fg.pw.radix, fg.pw.radix + fg.pw.nst), rh(fg.ph.radix, fg.ph.radix + fg.ph.nst);
    std::vector<HostCplx> twW, twH, tK1((size_t)M), tPair((size_t)M), tK2((size_t)M);
    stage_twiddles(W, rw, twW, fg.pw.off);
    stage_twiddles(H, rh, twH, fg.ph.off);
    parallel_for(H, [&](int64_t b, int64_t e) {
      for (int64_t k2 = b; k2 < e; ++k2)
        for (int m1 = 0; m1 < W; ++m1) {
          const HostCplx w = twM[(size_t)m1 * k2];   // m1 * k2 < M
          tK1[(size_t)m1 * H + k2] = w;
          tK2[(size_t)k2 * W + m1] = w;
          tPair[(size_t)k2 * W + m1] = pair_coeff(k2 + (int64_t)H * m1, M);
        }
    });
    pl->fg = fg;
    GL_TRY(dev_alloc(pl, &Z2, M));  // the row pass's output, column-major
    GL_TRY(dev_alloc(pl, &span, N));
    GL_TRY(dev_alloc(pl, &dtwW, twW.size()));
    GL_TRY(dev_alloc(pl, &dtwH, twH.size()));
    GL_TRY(dev_alloc(pl, &dK1, M));
    GL_TRY(dev_alloc(pl, &dPair, M));
    GL_TRY(dev_alloc(pl, &dK2, M));
    GL_TRYC(cudaMemcpyAsync(fl, fl_c.data(), N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(span, span_c.data(), N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dA, A_c.data(), sizeof(double) * N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dAi, Ai_c.data(), sizeof(double) * N, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dtwW, twW.data(), sizeof(DevCplx) * twW.size(), cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dtwH, twH.data(), sizeof(DevCplx) * twH.size(), cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dK1, tK1.data(), sizeof(DevCplx) * M, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dPair, tPair.data(), sizeof(DevCplx) * M, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaMemcpyAsync(dK2, tK2.data(), sizeof(DevCplx) * M, cudaMemcpyHostToDevice, pl->stream));
    GL_TRYC(cudaStreamSynchronize(pl->stream));  // host tables go out of scope
    a.W = W; a.H = H; a.G = 1; a.pw = pl->fg.pw; a.ph = pl->fg.ph; a.ls_col = fg.ls_col; a.ls_row = fg.ls_row;
    a.twW_n = (int)twW.size();
    // the row pass copies the whole table behind its four line buffers (unless it reads
    // the table through L1)
    if ((size_t)4 * fg.ls_row * 16 + (fg.row_var == 2 ? 0 : twW.size() * sizeof(DevCplx)) != fg.sm_row)
      GL_TRY(GL_ERR_SIZE);
    GL_TRYC(set_fused_smem_limits(fg));
    if (resident) {
      if (rg.twH_n != (int)twH.size() || rg.twW_n != (int)twW.size()) GL_TRY(GL_ERR_SIZE);
      pl->resident = true;
      pl->rg = rg;
    }
  }
  a.ll = ll; a.flags = fl; a.span = span; a.A = dA; a.Ainv = dAi; a.Z = Z; a.Z2 = Z2;
  a.twM = dtwM; a.twW = dtwW; a.twH = dtwH; a.twK1 = dK1; a.twPair = dPair; a.twK2 = dK2;
  a.digit = digit; a.hi = hi; a.status = status;
  *out = pl;
  int r = gl_reset(pl);
  if (r != GL_OK) {
    free_plan(pl);
    *out = nullptr;
    return r;
  }
  return GL_OK;
#undef GL_TRY
#undef GL_TRYC
}

extern "C" {

int gl_plan_describe(int p, int N, const gl_plan_opts* opts, gl_plan_info* info) {
  if (!info) return GL_ERR_ARG;
  gl_plan_opts o;
  if (opts) o = *opts;
  else gl_default_opts(&o);
  if (p < 3 || N < 16 || (N & 1) || N > p) return GL_ERR_ARG;
  if (o.mode != GL_MODE_FUSED && o.mode != GL_MODE_PLAIN) return GL_ERR_ARG;
  const int n = slice_depth(p, N);
  if (n < 0) return GL_ERR_RATIO;
  gl_plan tmp;
  tmp.p = p; tmp.N = N; tmp.M = N / 2; tmp.LO = p / N; tmp.n = n; tmp.mode = o.mode;
  if (o.cols_per_cta > 1) return GL_ERR_ARG;
  int sms = 0, ndev = 0;
  if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0 && o.device >= 0 && o.device < ndev)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o.device);
  if (sms <= 0) sms = 152;  // GB300
  if (o.batch_layout) sms = 1;
  int cap_c = kMaxRadix, cap_r = kMaxRadix;
  model_caps(tmp.M, o, o.batch_layout ? 1 : 0, &cap_c, &cap_r);
  int rc = o.mode == GL_MODE_FUSED ? choose_fused_geom(tmp.M, o.fft_h, sms, &tmp.fg, cap_c, cap_r)
                                   : choose_plain_geom(tmp.M, &tmp.pg);
  if (rc != GL_OK) return rc;
  tmp.device = -1;
  int r = gl_plan_get_info(&tmp, info);
  if (o.mode == GL_MODE_FUSED) {
    const size_t M = tmp.M, N8 = (size_t)N * 8;
    const size_t stages = (size_t)stage_offsets(tmp.fg.pw, tmp.fg.pw.off) + stage_offsets(tmp.fg.ph, tmp.fg.ph.off);
    info->device_bytes = N8 /*ll*/ + 2 * (size_t)N /*flags, span*/ + 2 * N8 /*A, Ainv*/ +
                         5 * M * 16 /*Z, Z2, 3 twiddle tables*/ + stages * 16 + (size_t)N * 5 /*digit, hi*/ +
                         sizeof(Status) + residue_scratch_bytes(N);
  }
  return r;
}

int gl_plan_destroy(gl_plan* plan) {
  if (!plan) return GL_ERR_ARG;
  free_plan(plan);
  return GL_OK;
}

int gl_plan_get_info(const gl_plan* pl, gl_plan_info* info) {
  if (!pl || !info) return GL_ERR_ARG;
  std::memset(info, 0, sizeof(*info));
  info->p = pl->p; info->N = pl->N;
  info->lo_bits = pl->LO; info->hi_bits = pl->LO + 1;
  info->carry_depth = pl->n; info->mode = pl->mode;
  if (pl->mode == GL_MODE_FUSED) {
    info->fft_w = pl->fg.W; info->fft_h = pl->fg.H; info->cols_per_cta = pl->fg.col_ws ? 2 : pl->fg.G;
    info->col_variant = !pl->fg.col_ip ? -1 : pl->fg.col_ws ? (pl->fg.col_pf ? 4 : 3) : (pl->fg.col_pf ? 2 : 1);
    info->row_variant = pl->fg.row_var ? pl->fg.row_var : -1;
    for (int i = 0; i < pl->fg.pw.nst; ++i) info->radix_w[i] = pl->fg.pw.radix[i];
    for (int i = 0; i < pl->fg.ph.nst; ++i) info->radix_h[i] = pl->fg.ph.radix[i];
    info->threads_col = pl->fg.t_col; info->threads_row = pl->fg.t_row;
    info->smem_col = (int)pl->fg.sm_col; info->smem_row = (int)pl->fg.sm_row;
  } else {
    info->fft_w = pl->M; info->fft_h = 1;
    for (int i = 0; i < pl->pg.nst && i < 8; ++i) info->radix_w[i] = pl->pg.radix[i];
  }
  info->device_bytes = pl->device_bytes;
  info->resident_ctas = pl->resident ? pl->rg.C : 0;
  info->resident_smem = pl->resident ? pl->rg.smem : 0;
  return GL_OK;
}

int gl_reset(gl_plan* pl) {
  if (!pl) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  GL_CUDA(launch_set_initial(pl->args, pl->mode, pl->stream));
  GL_CUDA(cudaMemsetAsync(pl->args.status, 0, sizeof(Status), pl->stream));
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  pl->iters_done = 0;
  pl->run_maxerr = 0.0;
  pl->from_state = false;
  pl->carry_valid = true;
  return GL_OK;
}

int gl_iterate(gl_plan* pl, int64_t iters, gl_iter_report* rep) {
  if (!pl || iters < 0) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  double call_max = 0.0;
  int status = GL_OK;
  int64_t done = 0;
  GL_CUDA(cudaEventRecord(pl->ev0, pl->stream));
  if (pl->mode == GL_MODE_PLAIN && !pl->carry_valid && iters > 0) {
    GL_CUDA(launch_dice(pl->args, pl->stream));
    pl->carry_valid = true;
  }
  while (done < iters) {
    const int64_t b = iters - done < pl->check_every ? iters - done : pl->check_every;
    int rc = enqueue(pl, b);
    if (rc != GL_OK) return rc;
    done += b;
    pl->iters_done += b;
    pl->carry_valid = pl->mode == GL_MODE_PLAIN;
    double e = 0.0;
    status = read_status(pl, &e);
    if (status == GL_ERR_CUDA) return status;
    if (e > call_max) call_max = e;
    if (status != GL_OK) break;
  }
  GL_CUDA(cudaEventRecord(pl->ev1, pl->stream));
  GL_CUDA(cudaEventSynchronize(pl->ev1));
  float ms = 0.f;
  GL_CUDA(cudaEventElapsedTime(&ms, pl->ev0, pl->ev1));
  if (rep) {
    rep->iterations = done;
    rep->total_iterations = pl->iters_done;
    rep->max_roundoff = call_max;
    rep->ms = ms;
    rep->status = status;
  }
  return status;
}

int gl_plan_stream(gl_plan* pl, void** cuda_stream) {
  if (!pl || !cuda_stream) return GL_ERR_ARG;
  *cuda_stream = (void*)pl->stream;
  return GL_OK;
}

int gl_enqueue(gl_plan* pl, int64_t iters) {
  if (!pl || iters < 0) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  if (pl->mode == GL_MODE_PLAIN && !pl->carry_valid && iters > 0) {
    GL_CUDA(launch_dice(pl->args, pl->stream));
    pl->carry_valid = true;
  }
  int rc = enqueue(pl, iters);
  if (rc != GL_OK) return rc;
  pl->iters_done += iters;
  if (iters > 0) pl->carry_valid = pl->mode == GL_MODE_PLAIN;
  return GL_OK;
}

int gl_sync_status(gl_plan* pl, gl_iter_report* rep) {
  if (!pl) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  double e = 0.0;
  int st = read_status(pl, &e);
  if (rep) {
    std::memset(rep, 0, sizeof(*rep));
    rep->total_iterations = pl->iters_done;
    rep->max_roundoff = e;
    rep->status = st;
  }
  return st;
}

int gl_launches_per_iteration(const gl_plan* pl) {
  if (!pl) return GL_ERR_ARG;
  if (pl->mode == GL_MODE_FUSED) return 3;
  return 2 * pl->pg.nst + 4;
}

int gl_profile_kernels(gl_plan* pl, int iters, double* ms_out, const char** names, int* nk) {
  if (!pl || !ms_out || iters < 1) return GL_ERR_ARG;
  if (pl->mode != GL_MODE_FUSED) return GL_ERR_STATE;
  GL_CUDA(cudaSetDevice(pl->device));
  static const char* kNames[3] = {"k_col_fwd", "k_row_sq", "k_col_inv"};
  if (pl->from_state) {  // consume a pending state load first
    int rc = launch_iterations(pl, 1);
    if (rc != GL_OK) return rc;
    pl->iters_done += 1;
  }
  cudaEvent_t ev[4];
  for (auto& e : ev) GL_CUDA(cudaEventCreate(&e));
  double acc[3] = {0, 0, 0};
  int rc = GL_OK;
  for (int it = 0; it < iters && rc == GL_OK; ++it) {
    for (int k = 0; k < 3; ++k) {
      if (cudaEventRecord(ev[k], pl->stream) != cudaSuccess) { rc = GL_ERR_CUDA; break; }
      if (launch_fused_kernel(pl->args, pl->fg, pl->stream, k) != cudaSuccess) { rc = GL_ERR_CUDA; break; }
    }
    if (rc != GL_OK) break;
    if (cudaEventRecord(ev[3], pl->stream) != cudaSuccess || cudaEventSynchronize(ev[3]) != cudaSuccess) {
      rc = GL_ERR_CUDA;
      break;
    }
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      acc[k] += ms;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc != GL_OK) return rc;
  pl->iters_done += iters;
  pl->carry_valid = false;
  for (int k = 0; k < 3; ++k) {
    ms_out[k] = acc[k] / iters;
    if (names) names[k] = kNames[k];
  }
  if (nk) *nk = 3;
  return GL_OK;
}

int gl_get_products(gl_plan* pl, int64_t* ll_out) {
  if (!pl || !ll_out) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  const long long* src = pl->args.ll;
  if (pl->mode == GL_MODE_FUSED) {  // un-permute into the (idle) work array
    long long* tmp = reinterpret_cast<long long*>(pl->args.Z);
    GL_CUDA(launch_permute_words(pl->args, pl->args.ll, tmp, false, pl->stream));
    src = tmp;
  }
  GL_CUDA(cudaMemcpyAsync(ll_out, src, sizeof(int64_t) * pl->N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  return GL_OK;
}

static int ensure_carry(gl_plan* pl) {
  if (!pl->carry_valid) {
    if (pl->mode == GL_MODE_FUSED) GL_CUDA(launch_dice_perm(pl->args, pl->stream));
    else GL_CUDA(launch_dice(pl->args, pl->stream));
    pl->carry_valid = true;
  }
  return GL_OK;
}

// The device address of pinned (page-locked, mapped) host memory, or null for any other
// pointer.
static void* mapped_host(const void* p) {
  cudaPointerAttributes at{};
  const bool ok = cudaPointerGetAttributes(&at, p) == cudaSuccess && at.type == cudaMemoryTypeHost;
  cudaGetLastError();  // a failed query leaves no error behind
  return ok ? at.devicePointer : nullptr;
}

// One host-state step of one fused iteration between pinned host buffers.  kind 1: the
// state as carry-added words (in[0] -> out[0]); kind 2: as the carry-save pair (digit
// in[0], carry in[1] -> out[0], out[1]).  out_dev: device addresses of the outputs'
// mappings.
struct HostStep {
  int kind;
  const void* in[2];
  void* out[2];
  void* out_dev[2];
};

// Copies in, the state-loading iteration, and the dicing, which also stores the state and
// the status into the mapped host buffers, so that transfer runs under the kernel instead
// of as copies after it.  Enqueued on the plan's stream (captured into a graph by the
// caller).
static cudaError_t enqueue_host_step(gl_plan* pl, const HostStep& hs, Status* status_dev) {
  const size_t N = (size_t)pl->N;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(pl->args.digit, hs.in[0], sizeof(int32_t) * N, cudaMemcpyHostToDevice, pl->stream)))
    return e;
  if (hs.kind == 1) e = cudaMemsetAsync(pl->args.hi, 0, N, pl->stream);
  else e = cudaMemcpyAsync(pl->args.hi, hs.in[1], N, cudaMemcpyHostToDevice, pl->stream);
  if (e) return e;
  if ((e = cudaMemsetAsync(pl->args.status, 0, sizeof(Status), pl->stream))) return e;
  if ((e = launch_fused_iteration(pl->args, pl->fg, pl->stream, true))) return e;
  if (hs.kind == 1) return launch_dice_words(pl->args, true, pl->stream, (int32_t*)hs.out_dev[0], status_dev);
  return launch_dice_perm(pl->args, pl->stream, (int*)hs.out_dev[0], (signed char*)hs.out_dev[1], status_dev);
}

// Whether this call runs as the captured step: one iteration of a fused (not resident)
// plan with graphs, every buffer pinned and mapped.  Fills hs->out_dev and *status_dev.
static bool host_step_mapped(gl_plan* pl, int64_t iters, HostStep* hs, Status** status_dev) {
  if (iters != 1 || pl->mode != GL_MODE_FUSED || pl->resident || !pl->use_graphs) return false;
  for (int i = 0; i < (hs->kind == 1 ? 1 : 2); ++i)
    if (!mapped_host(hs->in[i]) || !(hs->out_dev[i] = mapped_host(hs->out[i]))) return false;
  return (*status_dev = (Status*)mapped_host(pl->h_status)) != nullptr;
}

// Records the start event and launches the step as one graph (about ten calls fewer per
// step), built on the first call for these buffers and kept by the plan.
static int launch_host_step(gl_plan* pl, const HostStep& hs, Status* status_dev) {
  bool same = pl->hw_exec && pl->hw_kind == hs.kind;
  for (int i = 0; i < 2; ++i)
    same = same && pl->hw_in[i] == hs.in[i] && pl->hw_out[i] == hs.out[i] && pl->hw_out_dev[i] == hs.out_dev[i];
  if (!same) {
    if (pl->hw_exec) cudaGraphExecDestroy(pl->hw_exec);
    pl->hw_exec = nullptr;
    cudaGraph_t graph = nullptr;
    GL_CUDA(cudaStreamBeginCapture(pl->stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t es = enqueue_host_step(pl, hs, status_dev);
    const cudaError_t ec = cudaStreamEndCapture(pl->stream, &graph);
    if (es != cudaSuccess || ec != cudaSuccess || !graph) {
      if (graph) cudaGraphDestroy(graph);
      return GL_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&pl->hw_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      pl->hw_exec = nullptr;
      return GL_ERR_CUDA;
    }
    pl->hw_kind = hs.kind;
    for (int i = 0; i < 2; ++i) {
      pl->hw_in[i] = hs.in[i];
      pl->hw_out[i] = hs.out[i];
      pl->hw_out_dev[i] = hs.out_dev[i];
    }
  }
  GL_CUDA(cudaEventRecord(pl->ev0, pl->stream));
  GL_CUDA(cudaGraphLaunch(pl->hw_exec, pl->stream));
  pl->from_state = false;
  pl->iters_done += 1;
  pl->carry_valid = true;  // the device (digit, hi) is the state the host received
  return GL_OK;
}

// The end of a host-state call whose work is enqueued after ev0: wait for it, read the
// status it left in pl->h_status, report.
static int finish_host_step(gl_plan* pl, int64_t iters, gl_iter_report* rep) {
  GL_CUDA(cudaEventRecord(pl->ev1, pl->stream));
  GL_CUDA(cudaEventSynchronize(pl->ev1));
  const double e = std::ldexp((double)pl->h_status->maxerr64, -64);
  if (e > pl->run_maxerr) pl->run_maxerr = e;
  int st = GL_OK;
  if (pl->h_status->flags & kStatusTimeout) st = GL_ERR_TIMEOUT;
  else if (pl->h_status->flags) st = GL_ERR_OVERFLOW;
  else if (e >= pl->error_limit) st = GL_ERR_ROUNDOFF;
  float ms = 0.f;
  GL_CUDA(cudaEventElapsedTime(&ms, pl->ev0, pl->ev1));
  if (rep) {
    rep->iterations = iters;
    rep->total_iterations = pl->iters_done;
    rep->max_roundoff = e;
    rep->ms = ms;
    rep->status = st;
  }
  return st;
}

int gl_iterate_host(gl_plan* pl, const int32_t* digit_in, const int8_t* hi_in, int64_t iters, int32_t* digit_out,
                    int8_t* hi_out, gl_iter_report* rep) {
  if (!pl || !digit_in || !hi_in || !digit_out || !hi_out || iters < 0) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  const size_t N = (size_t)pl->N;
  HostStep hs{2, {digit_in, hi_in}, {digit_out, hi_out}, {nullptr, nullptr}};
  Status* status_dev = nullptr;
  if (host_step_mapped(pl, iters, &hs, &status_dev)) {
    const int rc = launch_host_step(pl, hs, status_dev);
    if (rc != GL_OK) return rc;
    return finish_host_step(pl, iters, rep);
  }
  GL_CUDA(cudaEventRecord(pl->ev0, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->args.digit, digit_in, sizeof(int32_t) * N, cudaMemcpyHostToDevice, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->args.hi, hi_in, N, cudaMemcpyHostToDevice, pl->stream));
  GL_CUDA(cudaMemsetAsync(pl->args.status, 0, sizeof(Status), pl->stream));
  pl->from_state = pl->mode == GL_MODE_FUSED;
  pl->carry_valid = true;
  if (iters > 0) {
    const int rc = enqueue(pl, iters);
    if (rc != GL_OK) return rc;
    pl->iters_done += iters;
    pl->carry_valid = pl->mode == GL_MODE_PLAIN;
  }
  const int rc = ensure_carry(pl);
  if (rc != GL_OK) return rc;
  GL_CUDA(cudaMemcpyAsync(digit_out, pl->args.digit, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaMemcpyAsync(hi_out, pl->args.hi, N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->h_status, pl->args.status, sizeof(Status), cudaMemcpyDeviceToHost, pl->stream));
  return finish_host_step(pl, iters, rep);
}

int gl_iterate_host_words(gl_plan* pl, const int32_t* words_in, int64_t iters, int32_t* words_out,
                          gl_iter_report* rep) {
  if (!pl || !words_in || !words_out || iters < 0) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  const size_t N = (size_t)pl->N;
  HostStep hs{1, {words_in, nullptr}, {words_out, nullptr}, {nullptr, nullptr}};
  Status* status_dev = nullptr;
  if (host_step_mapped(pl, iters, &hs, &status_dev)) {
    const int rc = launch_host_step(pl, hs, status_dev);
    if (rc != GL_OK) return rc;
    return finish_host_step(pl, iters, rep);
  }
  GL_CUDA(cudaEventRecord(pl->ev0, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->args.digit, words_in, sizeof(int32_t) * N, cudaMemcpyHostToDevice, pl->stream));
  GL_CUDA(cudaMemsetAsync(pl->args.hi, 0, N, pl->stream));
  GL_CUDA(cudaMemsetAsync(pl->args.status, 0, sizeof(Status), pl->stream));
  pl->from_state = pl->mode == GL_MODE_FUSED;
  pl->carry_valid = true;
  if (iters > 0) {
    const int rc = enqueue(pl, iters);
    if (rc != GL_OK) return rc;
    pl->iters_done += iters;
    pl->carry_valid = pl->mode == GL_MODE_PLAIN;
  }
  if (pl->carry_valid) GL_CUDA(launch_add_carry(pl->args, pl->stream));
  else GL_CUDA(launch_dice_words(pl->args, pl->mode == GL_MODE_FUSED, pl->stream));
  pl->carry_valid = true;  // (words, 0) is the carry-save state
  GL_CUDA(cudaMemcpyAsync(words_out, pl->args.digit, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->h_status, pl->args.status, sizeof(Status), cudaMemcpyDeviceToHost, pl->stream));
  return finish_host_step(pl, iters, rep);
}

int gl_get_carry_state(gl_plan* pl, int32_t* digit_out, int8_t* hi_out) {
  if (!pl || !digit_out || !hi_out) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  int rc = ensure_carry(pl);
  if (rc != GL_OK) return rc;
  GL_CUDA(cudaMemcpyAsync(digit_out, pl->args.digit, sizeof(int32_t) * pl->N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaMemcpyAsync(hi_out, pl->args.hi, pl->N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  return GL_OK;
}

int gl_set_products(gl_plan* pl, const int64_t* ll, int64_t iterations) {
  if (!pl || !ll || iterations < 0) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  if (pl->mode == GL_MODE_FUSED) {
    long long* tmp = reinterpret_cast<long long*>(pl->args.Z);
    GL_CUDA(cudaMemcpyAsync(tmp, ll, sizeof(int64_t) * pl->N, cudaMemcpyHostToDevice, pl->stream));
    GL_CUDA(launch_permute_words(pl->args, tmp, pl->args.ll, true, pl->stream));
  } else {
    GL_CUDA(cudaMemcpyAsync(pl->args.ll, ll, sizeof(int64_t) * pl->N, cudaMemcpyHostToDevice, pl->stream));
  }
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  pl->iters_done = iterations;
  pl->from_state = false;
  pl->carry_valid = false;
  return GL_OK;
}

int gl_set_carry_state(gl_plan* pl, const int32_t* digit, const int8_t* hi, int64_t iterations) {
  if (!pl || !digit || !hi || iterations < 0) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  GL_CUDA(cudaMemcpyAsync(pl->args.digit, digit, sizeof(int32_t) * pl->N, cudaMemcpyHostToDevice, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->args.hi, hi, pl->N, cudaMemcpyHostToDevice, pl->stream));
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  pl->iters_done = iterations;
  pl->from_state = pl->mode == GL_MODE_FUSED;
  pl->carry_valid = true;
  return GL_OK;
}

int gl_get_residue(gl_plan* pl, int32_t* digits_out, uint64_t* res64, int* is_zero) {
  if (!pl) return GL_ERR_ARG;
  GL_CUDA(cudaSetDevice(pl->device));
  int rc = ensure_carry(pl);
  if (rc != GL_OK) return rc;
  // the work array is idle between iterations: it holds the balanced digits
  int32_t* balanced = reinterpret_cast<int32_t*>(pl->args.Z);
  GL_CUDA(launch_residue(pl->args, pl->mode == GL_MODE_FUSED, balanced, pl->rscratch, pl->stream));
  GL_CUDA(cudaMemcpyAsync(pl->h_res, pl->rscratch + residue_head_offset(pl->N), sizeof(int32_t) * 69,
                          cudaMemcpyDeviceToHost, pl->stream));
  if (digits_out)
    GL_CUDA(cudaMemcpyAsync(digits_out, balanced, sizeof(int32_t) * pl->N, cudaMemcpyDeviceToHost, pl->stream));
  GL_CUDA(cudaStreamSynchronize(pl->stream));
  const int32_t* head = pl->h_res;
  const int32_t* scal = head + 64;
  const int flags = head[68];
  if (scal[2] != scal[3]) return GL_ERR_STATE;  // the end-around carry has no fixed point
  const bool all0 = !(flags & 1), allmax = !(flags & 2);
  // low 64 bits of the canonical digits; word j holds ceil(p(j+1)/N) - ceil(pj/N) bits
  uint64_t r = 0;
  int pos = 0;
  for (int j = 0; j < pl->N && j < 64 && pos < 64; ++j) {
    const int64_t lo = ((int64_t)pl->p * j + pl->N - 1) / pl->N;
    const int64_t hi = ((int64_t)pl->p * (j + 1) + pl->N - 1) / pl->N;
    r |= (uint64_t)(uint32_t)head[j] << pos;  // bits above 64 fall off
    pos += (int)(hi - lo);
  }
  if (allmax) r = 0;  // 2^p - 1 == 0
  if (res64) *res64 = r;
  if (is_zero) *is_zero = (all0 || allmax) ? 1 : 0;
  return GL_OK;
}

int gl_mersenne_test(gl_plan* pl, int64_t iters, gl_result* res) {
  if (!pl) return GL_ERR_ARG;
  const bool full = iters == 0;
  if (full) {
    int rc = gl_reset(pl);
    if (rc != GL_OK) return rc;
    iters = (int64_t)pl->p - 2;
  }
  gl_iter_report rep{};
  int st = gl_iterate(pl, iters, &rep);
  if (st == GL_ERR_CUDA || st == GL_ERR_ARG) return st;
  uint64_t r = 0;
  int z = 0;
  int rc = gl_get_residue(pl, nullptr, &r, &z);
  if (rc != GL_OK) return rc;
  if (res) {
    res->p = pl->p;
    res->N = pl->N;
    res->iterations = pl->iters_done;
    res->is_zero = z;
    res->is_prime = (pl->iters_done == (int64_t)pl->p - 2 && z && st == GL_OK) ? 1 : 0;
    res->res64 = r;
    res->max_roundoff = pl->run_maxerr;
    res->ms = rep.ms;
  }
  return st;
}

int gl_error_test(int p, int N, const gl_plan_opts* opts, int iters, gl_iter_report* rep) {
  gl_plan* pl = nullptr;
  int rc = gl_plan_create(p, N, opts, &pl);
  if (rc != GL_OK) return rc;
  if (iters <= 0) {
    iters = p / 10000;
    if (iters < 100) iters = 100;
    if (iters > 2500) iters = 2500;
  }
  rc = gl_iterate(pl, iters, rep);
  gl_plan_destroy(pl);
  return rc;
}

int gl_find_signal_size(int p, const gl_plan_opts* opts, int* N_out, double* ms_per_iter, double* max_roundoff) {
  if (!N_out || p < 64) return GL_ERR_ARG;
  gl_plan_opts o;
  if (opts) o = *opts;
  else gl_default_opts(&o);
  o.mode = GL_MODE_FUSED;
  o.fft_h = 0;
  o.error_limit = 0.5;
  o.check_every = 100;
  // candidate lengths, smallest first
  std::vector<int> cand;
  for (int64_t p2 = 2; p2 <= (1 << 26); p2 *= 2)
    for (int64_t p3 = 1, b = 0; b <= 5; p3 *= 3, ++b)
      for (int64_t p5 = 1, c = 0; c <= 3; p5 *= 5, ++c)
        for (int64_t p7 = 1, d = 0; d <= 2; p7 *= 7, ++d) {
          const int64_t N = p2 * p3 * p5 * p7;
          if (N < 64 || N > p / 8 || N > (1 << 27)) continue;
          if (slice_depth(p, (int)N) < 0) continue;
          cand.push_back((int)N);
        }
  std::sort(cand.begin(), cand.end());
  cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  int best = 0, first = 0;
  double best_ms = 1e300, best_err = 0.0;
  for (int N : cand) {
    if (first && N > first + first / 7) break;  // within ~15 % of the smallest accepted
    gl_plan* pl = nullptr;
    int rc = gl_plan_create(p, N, &o, &pl);
    if (rc == GL_ERR_NOMEM || rc == GL_ERR_NODEVICE || rc == GL_ERR_CUDA) return rc;
    if (rc != GL_OK) continue;
    gl_iter_report rep{};
    rc = gl_iterate(pl, 100, &rep);
    double ms = -1.0;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, pl->device);
    autotune_layout(N / 2, pl->n, sms, 0, &ms);
    gl_plan_destroy(pl);
    if (rc == GL_ERR_CUDA) return rc;
    if (rc != GL_OK || rep.max_roundoff >= 0.30 || ms <= 0.0) continue;
    if (!first) first = N;
    if (ms < best_ms) {
      best_ms = ms;
      best = N;
      best_err = rep.max_roundoff;
    }
  }
  if (!best) return GL_ERR_SIZE;
  *N_out = best;
  if (ms_per_iter) *ms_per_iter = best_ms;
  if (max_roundoff) *max_roundoff = best_err;
  return GL_OK;
}

float errorTest(int testPrime, int signalSize) {
  gl_iter_report rep{};
  int rc = gl_error_test(testPrime, signalSize, nullptr, 0, &rep);
  if (rc != GL_OK || rep.iterations <= 0) return -1.0f;
  return (float)(rep.ms / (double)rep.iterations);
}

int mersenneTest(int testPrime, int signalSize) {
  gl_plan* pl = nullptr;
  int rc = gl_plan_create(testPrime, signalSize, nullptr, &pl);
  if (rc != GL_OK) return rc;
  gl_result res{};
  rc = gl_mersenne_test(pl, 0, &res);
  gl_plan_destroy(pl);
  if (rc != GL_OK) return rc;
  if (res.is_prime)
    std::printf("M( %d )P, n = %d, gpulucas_gb300 v%d.%d.%d\n", testPrime, signalSize, 0, 1, 0);
  else
    std::printf("M( %d )C, 0x%016llx, n = %d, gpulucas_gb300 v%d.%d.%d\n", testPrime,
                (unsigned long long)res.res64, signalSize, 0, 1, 0);
  std::fflush(stdout);
  return res.is_prime;
}

int gl_selftest_bounded_wait(int device, int tries) {
  if (tries < 1) return GL_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GL_ERR_NODEVICE;
  if (device < 0 || device >= ndev || cudaSetDevice(device) != cudaSuccess) return GL_ERR_ARG;
  Status* d = nullptr;
  Status h{};
  if (cudaMalloc(&d, sizeof(Status)) != cudaSuccess) return GL_ERR_NOMEM;
  int rc = GL_OK;
  if (cudaMemset(d, 0, sizeof(Status)) != cudaSuccess || launch_wait_selftest(d, tries, 0) != cudaSuccess ||
      cudaMemcpy(&h, d, sizeof(Status), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = GL_ERR_CUDA;
  cudaFree(d);
  if (rc != GL_OK) return rc;
  return (h.flags & kStatusTimeout) ? GL_ERR_TIMEOUT : GL_OK;
}

// Runs probe(blocks, threads, iters) with iters doubling until one launch takes >= ms;
// returns its milliseconds and the iteration count.
}  // extern "C"
template <typename Probe>
static int timed_probe(int device, double ms, Probe probe, float* el_out, long long* iters_out, int* blocks_out) {
  GL_CUDA(cudaSetDevice(device));
  int nsm = 0;
  GL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  const int threads = 256, blocks = nsm * 4;
  double* buf = nullptr;
  GL_CUDA(cudaMalloc(&buf, sizeof(double) * threads * blocks));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  long long iters = 1024;
  float el = 0.f;
  int rc = GL_OK;
  for (int rep = 0; rep < 12; ++rep) {
    cudaEventRecord(a, 0);
    if (probe(blocks, threads, iters, buf, (cudaStream_t)0) != cudaSuccess) { rc = GL_ERR_CUDA; break; }
    cudaEventRecord(b, 0);
    if (cudaEventSynchronize(b) != cudaSuccess) { rc = GL_ERR_CUDA; break; }
    cudaEventElapsedTime(&el, a, b);
    if (el >= ms) break;
    iters *= 2;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  *el_out = el;
  *iters_out = iters;
  *blocks_out = blocks;
  return rc;
}
extern "C" {

int gl_probe_fp64_peak(int device, double ms, double* tflops) {
  if (!tflops || ms <= 0) return GL_ERR_ARG;
  float el = 0.f;
  long long iters = 0;
  int blocks = 0;
  const int rc = timed_probe(device, ms, probe_fp64, &el, &iters, &blocks);
  if (rc == GL_OK) {
    const double fmas = (double)blocks * 256 * 8.0 * (double)iters;
    *tflops = 2.0 * fmas / (el * 1e-3) / 1e12;
  }
  return rc;
}

int gl_probe_fp64_butterfly(int device, double ms, double* instr_per_s) {
  if (!instr_per_s || ms <= 0) return GL_ERR_ARG;
  float el = 0.f;
  long long iters = 0;
  int blocks = 0;
  const int rc = timed_probe(device, ms, probe_butterfly, &el, &iters, &blocks);
  if (rc == GL_OK) *instr_per_s = (double)blocks * 256 * kProbeButterflyInstr * (double)iters / (el * 1e-3);
  return rc;
}

}  // extern "C"
