// gl_batch.cpp -- many Lucas-Lehmer tests advanced together.
//
// Each test keeps a fused-form plan (its own tables and buffers, layout chosen for
// total work since the batch, not the test, fills the device).  The batch uploads a
// descriptor table of every test's iteration arguments and two unit maps -- one entry
// per column (column passes) and per row pair (row pass), ordered longest unit first
// -- so one set of three launches advances every test by one iteration.  Batches of
// 64 iterations are replayed from one CUDA graph.  Each test's round-off status word
// lives in one contiguous array read back with a single copy.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gl_internal.h"
#include "gl_plan.h"
#include "gl_tables.h"

using namespace gl;

struct gl_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<gl_plan*> plans;
  bool owns_plans = true;
  // row-pass units of several row pairs for short-row members (gl_batch_create).  Off for
  // batches over existing plans (the server's lanes): they share the device with
  // higher-priority lanes, and longer-running CTAs there hold SMs the lead lane waits for
  // (served p99 85.6 -> 91.7 s measured with them on)
  bool merge_row_pairs = true;
  std::vector<void*> allocs;
  BatchLaunch launch{};
  Status* d_status = nullptr;
  std::vector<Status> h_status;
  std::vector<double> maxerr;  // per test, over the run
  int64_t iters_done = 0;
  int check_every = 1000;
  double error_limit = 0.4;
  cudaGraphExec_t gexec = nullptr;
  size_t device_bytes = 0;
};

namespace {

constexpr int kBatchGraph = 64;

void free_batch(gl_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  for (void* p : b->allocs) cudaFree(p);
  if (b->stream) cudaStreamDestroy(b->stream);
  if (b->owns_plans)
    for (gl_plan* p : b->plans) gl_plan_destroy(p);
  delete b;
}

template <typename T>
int upload(gl_batch* b, T** dst, const std::vector<T>& v) {
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(1, v.size())) != cudaSuccess) return GL_ERR_NOMEM;
  b->allocs.push_back(p);
  b->device_bytes += sizeof(T) * v.size();
  if (!v.empty() && (cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, b->stream) !=
                         cudaSuccess ||
                     cudaStreamSynchronize(b->stream) != cudaSuccess))
    return GL_ERR_CUDA;
  *dst = static_cast<T*>(p);
  return GL_OK;
}

int launch_n(gl_batch* b, int64_t k) {
  for (int64_t i = 0; i < k; ++i)
    if (launch_batch_iteration(b->launch, b->stream, false) != cudaSuccess) return GL_ERR_CUDA;
  return GL_OK;
}

int enqueue(gl_batch* b, int64_t k) {
  if (k >= kBatchGraph) {
    if (!b->gexec) {
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GL_ERR_CUDA;
      const int rc = launch_n(b, kBatchGraph);
      const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
      if (rc != GL_OK || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return GL_ERR_CUDA;
      }
      const cudaError_t ei = cudaGraphInstantiate(&b->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) {
        b->gexec = nullptr;
        return GL_ERR_CUDA;
      }
    }
    while (k >= kBatchGraph) {
      if (cudaGraphLaunch(b->gexec, b->stream) != cudaSuccess) return GL_ERR_CUDA;
      k -= kBatchGraph;
    }
  }
  return launch_n(b, k);
}

// Reads every test's status; returns the worst status and the max round-off.
int read_status(gl_batch* b, double* worst_err) {
  const size_t n = b->plans.size();
  if (cudaMemcpyAsync(b->h_status.data(), b->d_status, sizeof(Status) * n, cudaMemcpyDeviceToHost, b->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return GL_ERR_CUDA;
  int st = GL_OK;
  double worst = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double e = std::ldexp((double)b->h_status[i].maxerr64, -64);
    b->maxerr[i] = std::max(b->maxerr[i], e);
    worst = std::max(worst, e);
    if (b->h_status[i].flags & kStatusTimeout) st = GL_ERR_TIMEOUT;
    else if (b->h_status[i].flags && st != GL_ERR_TIMEOUT) st = GL_ERR_OVERFLOW;
    else if (e >= b->error_limit && st == GL_OK) st = GL_ERR_ROUNDOFF;
  }
  if (worst_err) *worst_err = worst;
  return st;
}

// Row pairs per row-pass unit of a batch member: at most this many, within this much
// shared memory per CTA (the unit's line buffers and stage values)
constexpr int kMaxRowPairsPerUnit = 8;
constexpr size_t kRowUnitSmem = 48 * 1024;
constexpr int kRowUnitsPerSM = 16;

// descriptor table, status array and unit maps of the batch's plans
int assemble(gl_batch* b) {
  const int ntests = (int)b->plans.size();
#define GB_TRY(x)      \
  do {                 \
    int r_ = (x);      \
    if (r_ != GL_OK) { \
      return r_;       \
    }                  \
  } while (0)
  // per-test status words, one contiguous array
  std::vector<Status> zero((size_t)ntests);
  std::memset(zero.data(), 0, sizeof(Status) * zero.size());
  GB_TRY(upload(b, &b->d_status, zero));
  b->h_status.resize((size_t)ntests);
  b->maxerr.assign((size_t)ntests, 0.0);
  std::vector<IterArgs> desc((size_t)ntests);
  int t_col = 64, t_row = 64;
  size_t sm_col = 0, sm_row = 0;
  for (int i = 0; i < ntests; ++i) {
    desc[i] = b->plans[i]->args;
    desc[i].status = b->d_status + i;
    t_col = std::max(t_col, b->plans[i]->fg.t_col);
    t_row = std::max(t_row, b->plans[i]->fg.t_row);
    // the batched column kernels always use the two-buffer line DFT
    sm_col = std::max(sm_col, (size_t)2 * b->plans[i]->fg.ls_col * 16);
    sm_row = std::max(sm_row, b->plans[i]->fg.sm_row);
  }
  IterArgs* d_desc = nullptr;
  GB_TRY(upload(b, &d_desc, desc));
  // unit maps, longest units first so the tail of each launch is short work
  std::vector<int> order((size_t)ntests);
  for (int i = 0; i < ntests; ++i) order[i] = i;
  std::vector<int2> cols, rows;
  std::sort(order.begin(), order.end(), [&](int a, int c) {
    return gl_plan_unit_cost(b->plans[a], false) > gl_plan_unit_cost(b->plans[c], false);
  });
  for (int t : order)
    for (int u = 0; u < b->plans[t]->fg.W; ++u) cols.push_back(make_int2(t, u));
  // row units of k row pairs: as many pairs as the block takes in one round of the widest
  // stage (the most butterflies), at most 8 and within kRowUnitSmem of shared memory, and
  // only while the batch keeps kRowUnitsPerSM units per SM (a batch of a few tests needs
  // one pair per CTA to spread its rows over the device)
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess || sms < 1) {
    cudaGetLastError();
    sms = 152;
  }
  long total_pairs = 0;
  for (int i = 0; i < ntests; ++i) total_pairs += b->plans[i]->fg.H / 2 + 1;
  const int kcap = b->merge_row_pairs ? (int)std::max(1L, std::min((long)kMaxRowPairsPerUnit,
                                                                 total_pairs / ((long)kRowUnitsPerSM * sms)))
                                     : 1;
  std::vector<int> pairs((size_t)ntests, 1);
  sm_row = 0;
  for (int i = 0; i < ntests; ++i) {
    const FusedGeom& g = b->plans[i]->fg;
    int widest = 1;
    for (int s = 0; s < g.pw.nst; ++s) widest = std::max(widest, 2 * g.W / g.pw.radix[s]);
    const size_t lines = (size_t)4 * g.ls_row * 16, stage = g.sm_row - lines;
    int k = std::max(1, std::min(kcap, t_row / widest));
    while (k > 1 && (size_t)k * lines + stage > kRowUnitSmem) --k;
    pairs[(size_t)i] = k;
    sm_row = std::max(sm_row, (size_t)k * lines + stage);
  }
  std::sort(order.begin(), order.end(), [&](int a, int c) {
    return gl_plan_unit_cost(b->plans[a], true) * pairs[(size_t)a] >
           gl_plan_unit_cost(b->plans[c], true) * pairs[(size_t)c];
  });
  for (int t : order) {
    const int last = b->plans[t]->fg.H / 2, k = pairs[(size_t)t];
    for (int c = 0; c <= last; c += k) rows.push_back(make_int2(t, c | (std::min(k, last + 1 - c) << 20)));
  }
  int2 *d_cols = nullptr, *d_rows = nullptr;
  GB_TRY(upload(b, &d_cols, cols));
  GB_TRY(upload(b, &d_rows, rows));
  b->launch.tests = d_desc;
  b->launch.col_units = d_cols;
  b->launch.row_units = d_rows;
  b->launch.ncol = (int)cols.size();
  b->launch.nrow = (int)rows.size();
  b->launch.t_col = t_col;
  b->launch.t_row = t_row;
  b->launch.sm_col = sm_col;
  b->launch.sm_row = sm_row;
  GB_TRY(set_batch_smem_limits() == cudaSuccess ? GL_OK : GL_ERR_CUDA);
#undef GB_TRY
  return GL_OK;
}

// smallest even N >= 64 with N/2 7-smooth, a carry depth for p/N, and p/N <= bits(N)
template <typename Bits>
int smallest_length(int p, Bits bits, int* N_out) {
  const int64_t cap = 1 << 27;
  int best = 0;
  for (int64_t p2 = 2; p2 <= cap; p2 *= 2)
    for (int64_t p3 = p2; p3 <= cap; p3 *= 3)
      for (int64_t p5 = p3; p5 <= cap; p5 *= 5)
        for (int64_t N = p5; N <= cap; N *= 7) {
          if (N < 64 || (double)p / (double)N > bits((double)N)) continue;
          if (slice_depth(p, (int)N) < 0) continue;
          if (!best || N < best) best = (int)N;
        }
  if (!best) return GL_ERR_SIZE;
  *N_out = best;
  return GL_OK;
}

// status of one test from the last status read
int test_status_of(const gl_batch* b, int index) {
  const unsigned fl = b->h_status[(size_t)index].flags;
  if (fl & kStatusTimeout) return GL_ERR_TIMEOUT;
  if (fl) return GL_ERR_OVERFLOW;
  return b->maxerr[(size_t)index] >= b->error_limit ? GL_ERR_ROUNDOFF : GL_OK;
}

}  // namespace

extern "C" {

int gl_smallest_signal_size(int p, double max_bits_per_word, int* N_out) {
  if (!N_out || p < 64 || !(max_bits_per_word > 1.0)) return GL_ERR_ARG;
  return smallest_length(p, [&](double) { return max_bits_per_word; }, N_out);
}

int gl_safe_signal_size(int p, int* N_out) {
  if (!N_out || p < 64) return GL_ERR_ARG;
  return smallest_length(p, [](double N) { return 19.2 - 0.26 * std::log2(N / 163840.0); }, N_out);
}

int gl_fast_signal_size(int p, double slack, int* N_out) {
  if (!N_out || p < 64 || !(slack >= 0.0)) return GL_ERR_ARG;
  int N0 = 0;
  const int rc = gl_safe_signal_size(p, &N0);
  if (rc != GL_OK) return rc;
  const int64_t top = (int64_t)((double)N0 * (1.0 + slack));
  // Measured on GB300 (one test alone, timed layout): lengths whose odd part is 1 or 3
  // run markedly faster than their neighbours (98304 = 2^15 3: 33 us per iteration;
  // 84672, 86016, 87480, 90000, 92160, 96000, 100352: 39-43 us), because every line
  // plan is then radix 4/8 with at most one radix-3 stage.  The smallest such length
  // within the slack wins; otherwise the cost model picks.
  int best = N0;
  double best_cost = gl_model_iteration_cost(N0 / 2, 152);
  int pow2ish = 0;
  for (int64_t p2 = 2; p2 <= top; p2 *= 2)
    for (int64_t p3 = p2; p3 <= top; p3 *= 3)
      for (int64_t p5 = p3; p5 <= top; p5 *= 5)
        for (int64_t N = p5; N <= top; N *= 7) {
          if (N < N0 || slice_depth(p, (int)N) < 0) continue;
          int64_t odd = N;
          while (!(odd & 1)) odd >>= 1;
          if ((odd == 1 || odd == 3) && (!pow2ish || N < pow2ish)) pow2ish = (int)N;
          if (N == N0) continue;
          const double c = gl_model_iteration_cost((int)(N / 2), 152);
          if (c < best_cost) {
            best_cost = c;
            best = (int)N;
          }
        }
  *N_out = pow2ish ? pow2ish : best;
  return GL_OK;
}

int gl_batch_create(const int* p, const int* N, int ntests, const gl_plan_opts* opts, gl_batch** out) {
  if (!p || !out || ntests < 1) return GL_ERR_ARG;
  *out = nullptr;
  gl_plan_opts o;
  if (opts) o = *opts;
  else gl_default_opts(&o);
  o.mode = GL_MODE_FUSED;
  o.autotune = 0;
  o.fft_h = 0;
  gl_batch* b = new gl_batch();
  b->device = o.device;
  b->check_every = o.check_every;
  b->error_limit = o.error_limit;
#define GB_TRY(x)      \
  do {                 \
    int r_ = (x);      \
    if (r_ != GL_OK) { \
      free_batch(b);   \
      return r_;       \
    }                  \
  } while (0)
  if (cudaSetDevice(o.device) != cudaSuccess) {
    delete b;
    return GL_ERR_NODEVICE;
  }
  GB_TRY(gl_make_stream(&b->stream, o.high_priority) == cudaSuccess ? GL_OK : GL_ERR_CUDA);
  for (int i = 0; i < ntests; ++i) {
    int n_i = N ? N[i] : 0;
    if (n_i == 0) GB_TRY(gl_smallest_signal_size(p[i], 19.5, &n_i));
    gl_plan* pl = nullptr;
    GB_TRY(gl_plan_create_ex(p[i], n_i, &o, 1, &pl));
    b->plans.push_back(pl);
    b->device_bytes += pl->device_bytes;
  }
  GB_TRY(assemble(b));
#undef GB_TRY
  *out = b;
  return GL_OK;
}

int gl_batch_create_from_plans(gl_plan* const* plans, int nplans, const gl_plan_opts* opts, gl_batch** out) {
  if (!plans || !out || nplans < 1) return GL_ERR_ARG;
  *out = nullptr;
  gl_plan_opts o;
  if (opts) o = *opts;
  else gl_default_opts(&o);
  for (int i = 0; i < nplans; ++i)
    if (!plans[i] || plans[i]->mode != GL_MODE_FUSED || plans[i]->device != plans[0]->device) return GL_ERR_ARG;
  // a pending state load (after gl_set_carry_state / gl_plan_resume) is consumed by the
  // plan's own next iteration; the batch's kernels start from the products
  for (int i = 0; i < nplans; ++i)
    if (plans[i]->from_state) return GL_ERR_STATE;
  gl_batch* b = new gl_batch();
  b->owns_plans = false;
  b->merge_row_pairs = false;
  b->device = plans[0]->device;
  b->check_every = o.check_every;
  b->error_limit = o.error_limit;
  if (cudaSetDevice(b->device) != cudaSuccess ||
      gl_make_stream(&b->stream, o.high_priority) != cudaSuccess) {
    free_batch(b);
    return GL_ERR_CUDA;
  }
  for (int i = 0; i < nplans; ++i) {
    b->plans.push_back(plans[i]);
    // the batch's kernels must see each plan's pending work
    if (cudaStreamSynchronize(plans[i]->stream) != cudaSuccess) {
      free_batch(b);
      return GL_ERR_CUDA;
    }
  }
  const int rc = assemble(b);
  if (rc != GL_OK) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return GL_OK;
}

int gl_batch_destroy(gl_batch* b) {
  if (!b) return GL_ERR_ARG;
  free_batch(b);
  return GL_OK;
}

int gl_batch_stream(gl_batch* b, void** stream) {
  if (!b || !stream) return GL_ERR_ARG;
  *stream = (void*)b->stream;
  return GL_OK;
}

int gl_batch_enqueue(gl_batch* b, int64_t iters) {
  if (!b || iters < 0) return GL_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return GL_ERR_CUDA;
  const int rc = enqueue(b, iters);
  if (rc != GL_OK) return rc;
  b->iters_done += iters;
  for (gl_plan* p : b->plans) gl_plan_note_external_iterations(p, iters);
  return GL_OK;
}

int gl_batch_iterate(gl_batch* b, int64_t iters, gl_iter_report* rep) {
  if (!b || iters < 0) return GL_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return GL_ERR_CUDA;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return GL_ERR_CUDA;
  cudaEventRecord(e0, b->stream);
  int64_t done = 0;
  int st = GL_OK;
  double worst = 0.0;
  while (done < iters) {
    const int64_t k = std::min<int64_t>(iters - done, b->check_every);
    st = gl_batch_enqueue(b, k);
    if (st != GL_OK) break;
    done += k;
    double e = 0.0;
    st = read_status(b, &e);
    worst = std::max(worst, e);
    if (st != GL_OK) break;
  }
  cudaEventRecord(e1, b->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rep) {
    rep->iterations = done;
    rep->total_iterations = b->iters_done;
    rep->max_roundoff = worst;
    rep->ms = ms;
    rep->status = st;
  }
  return st;
}

int gl_batch_sync_status(gl_batch* b, gl_iter_report* rep) {
  if (!b) return GL_ERR_ARG;
  double e = 0.0;
  const int st = read_status(b, &e);
  if (rep) {
    std::memset(rep, 0, sizeof(*rep));
    rep->total_iterations = b->iters_done;
    rep->max_roundoff = e;
    rep->status = st;
  }
  return st;
}

int gl_batch_query(gl_batch* b) {
  if (!b) return GL_ERR_ARG;
  const cudaError_t e = cudaStreamQuery(b->stream);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return GL_ERR_CUDA;
}

int gl_batch_result(gl_batch* b, int index, gl_result* r, int* status) {
  if (!b || !r || index < 0 || index >= (int)b->plans.size()) return GL_ERR_ARG;
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return GL_ERR_CUDA;
  gl_plan* pl = b->plans[(size_t)index];
  uint64_t res = 0;
  int z = 0;
  const int rc = gl_get_residue(pl, nullptr, &res, &z);
  if (rc != GL_OK) return rc;
  std::memset(r, 0, sizeof(*r));
  r->p = pl->p;
  r->N = pl->N;
  r->iterations = pl->iters_done;
  r->is_zero = z;
  r->is_prime = (pl->iters_done == (int64_t)pl->p - 2 && z) ? 1 : 0;
  r->res64 = res;
  r->max_roundoff = b->maxerr[(size_t)index];
  if (status) *status = test_status_of(b, index);
  return GL_OK;
}

int gl_batch_test_status(const gl_batch* b, int index, double* max_roundoff, int* status) {
  if (!b || index < 0 || index >= (int)b->plans.size()) return GL_ERR_ARG;
  const double e = b->maxerr[(size_t)index];
  if (max_roundoff) *max_roundoff = e;
  if (status) *status = test_status_of(b, index);
  return GL_OK;
}

int gl_batch_get_info(const gl_batch* b, gl_batch_info* info) {
  if (!b || !info) return GL_ERR_ARG;
  std::memset(info, 0, sizeof(*info));
  info->ntests = (int)b->plans.size();
  info->col_units = b->launch.ncol;
  info->row_units = b->launch.nrow;
  info->threads_col = b->launch.t_col;
  info->threads_row = b->launch.t_row;
  info->smem_col = (int)b->launch.sm_col;
  info->smem_row = (int)b->launch.sm_row;
  info->device_bytes = b->device_bytes;
  info->iterations = b->iters_done;
  return GL_OK;
}

int gl_batch_test_info(const gl_batch* b, int index, gl_plan_info* info) {
  if (!b || index < 0 || index >= (int)b->plans.size()) return GL_ERR_ARG;
  return gl_plan_get_info(b->plans[(size_t)index], info);
}

}  // extern "C"
