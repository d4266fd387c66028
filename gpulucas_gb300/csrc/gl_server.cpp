// gl_server.cpp -- request loop with continuous batching (gl_server_* in gpulucas.h).
//
// One background thread runs the loop; plan building runs on a small pool of worker
// threads.  The loop, each turn:
//   1. takes newly submitted requests, sizes them (signal_size, footprint);
//   2. admits queued requests in arrival order while the slot limit and the HBM budget
//      allow, handing each to the builders (a request that can never fit is rejected
//      once nothing else is live);
//   3. moves built tests into their lane (chain: full tests and long requests; bulk:
//      the rest) and keeps the chain test with the most iterations left alone in the
//      lead lane (highest stream priority), so the longest dependent chain runs at its
//      own speed while everything else fills the rest of the device;
//   4. for each lane: if its step has finished, reads every test's round-off and status,
//      records checkpoints, retires finished or failed tests (a round-off failure
//      re-queues the request at the next larger length while retries remain) and drops
//      the batch if its membership changed; if the lane is idle and has live tests,
//      rebuilds the batch when needed and enqueues the next step: at most step_ms of
//      GPU time (from the last measured step), never past the next completion or
//      checkpoint of its tests.
// Steps are enqueued asynchronously and polled, so the lanes' streams stay busy while
// the host sizes, admits and retires.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "gl_plan.h"
#include "gpulucas.h"

namespace {

using Clock = std::chrono::steady_clock;

double flop_alg(int N) { return 5.0 * N * std::log2((double)N) + 4.0 * N; }

// ---------------------------------------------------------------------------
// the library's own plans and batches
struct GpuEngine {
  int device = 0;
  double error_limit = 0.4;
  int check_every = 1000;
};

gl_plan_opts engine_opts(const GpuEngine* g) {
  gl_plan_opts o;
  gl_default_opts(&o);
  o.device = g->device;
  o.autotune = 0;
  o.batch_layout = 0;  // each test keeps its own best layout: a test left alone is not slowed
  o.error_limit = g->error_limit;
  o.check_every = g->check_every;
  return o;
}

int ge_signal_size(void*, int p, double bits, int above, int* N) {
  if (above) return gl_smallest_signal_size(p, (double)p / (above + 1.0), N);
  if (bits > 0.0) return gl_smallest_signal_size(p, bits, N);
  return gl_fast_signal_size(p, 0.2, N);
}
int ge_footprint(void* ctx, int p, int N, size_t* bytes) {
  gl_plan_opts o = engine_opts(static_cast<GpuEngine*>(ctx));
  gl_plan_info info;
  const int rc = gl_plan_describe(p, N, &o, &info);
  if (rc == GL_OK) *bytes = info.device_bytes;
  return rc;
}
int ge_create(void* ctx, int p, int N, void** test) {
  gl_plan_opts o = engine_opts(static_cast<GpuEngine*>(ctx));
  gl_plan* pl = nullptr;
  const int rc = gl_plan_create(p, N, &o, &pl);  // starts from S0 = 4
  *test = pl;
  return rc;
}
void ge_destroy(void*, void* test) { gl_plan_destroy(static_cast<gl_plan*>(test)); }
int ge_batch(void* ctx, void* const* tests, int n, int high, void** batch) {
  gl_plan_opts o = engine_opts(static_cast<GpuEngine*>(ctx));
  o.high_priority = high;
  gl_batch* b = nullptr;
  const int rc = gl_batch_create_from_plans(reinterpret_cast<gl_plan* const*>(tests), n, &o, &b);
  *batch = b;
  return rc;
}
void ge_close_batch(void*, void* batch) { gl_batch_destroy(static_cast<gl_batch*>(batch)); }
int ge_start(void*, void* batch, int64_t iters) { return gl_batch_enqueue(static_cast<gl_batch*>(batch), iters); }
int ge_ready(void*, void* batch) { return gl_batch_query(static_cast<gl_batch*>(batch)); }
int ge_finish(void*, void* batch, int n, double* err, int* st) {
  gl_batch* b = static_cast<gl_batch*>(batch);
  const int rc = gl_batch_sync_status(b, nullptr);
  if (rc == GL_ERR_CUDA || rc == GL_ERR_ARG) return rc;
  for (int i = 0; i < n; ++i) {
    const int r = gl_batch_test_status(b, i, err + i, st + i);
    if (r != GL_OK) return r;
  }
  return GL_OK;
}
int ge_res64(void*, void* test, uint64_t* res64, int* zero) {
  return gl_get_residue(static_cast<gl_plan*>(test), nullptr, res64, zero);
}

// ---------------------------------------------------------------------------
struct Request {
  int64_t id = 0;
  int p = 0;
  int64_t iterations = 0;
  bool full = false;
  double arrival = 0.0;
};

struct Live {
  Request r;
  int N = 0;
  size_t bytes = 0;
  double admit = 0.0;
  void* test = nullptr;
  int build_rc = GL_OK;
  int64_t done = 0;
  double maxerr = 0.0;
  int attempts = 1;
  std::vector<std::pair<int64_t, uint64_t>> checkpoints;
};

struct Lane {
  int level = 0;          // stream priority level (gl_plan_opts.high_priority)
  std::vector<Live*> live;
  void* batch = nullptr;
  std::vector<Live*> members;
  double iter_ms = 0.0;   // measured ms per iteration of the current members, 0 = unknown
  int64_t inflight = 0;
  Clock::time_point t_start;
  double busy_s = 0.0;
  int64_t steps = 0, rebuilds = 0;
  int peak_live = 0;
};

}  // namespace

struct gl_server {
  gl_server_opts o{};
  gl_server_engine eng{};
  GpuEngine gpu;
  Clock::time_point t0;

  std::mutex mu;                  // guards everything below up to `loop state`
  std::condition_variable cv;     // submissions, completions, builds, stop
  std::deque<Request> submitted;
  std::deque<gl_completion> completions;
  std::map<int64_t, std::vector<std::pair<int64_t, uint64_t>>> checkpoints;
  std::deque<Live*> to_build;
  std::vector<Live*> built;
  int64_t n_submitted = 0, n_completed = 0;
  bool stop = false;
  int error = GL_OK;
  gl_server_stats stats{};

  // loop state (loop thread only)
  std::deque<Live*> queue;
  int building = 0;
  Lane lanes[3];
  int nlanes = 3;
  size_t used = 0;

  std::thread loop_thread;
  std::vector<std::thread> builders;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Lanes: with three, 0 = lead (the chain test with the most iterations left, alone, at
// the highest priority), 1 = chain (the other long tests), 2 = bulk; with two, 0 = chain,
// 1 = bulk; with one, everything in lane 0.
int lane_of(const gl_server* s, const Request& r) {
  if (s->nlanes == 1) return 0;
  const bool chain = r.full || r.iterations > s->o.chain_iterations;
  return chain ? s->nlanes - 2 : s->nlanes - 1;
}

// Three lanes: keep the chain test with the most iterations left alone in the lead lane.
// Moves happen only while both lanes are idle; returns true if a move is pending.
bool promote(gl_server* s) {
  if (s->nlanes != 3) return false;
  Lane& L = s->lanes[0];
  Lane& C = s->lanes[1];
  Live* best = nullptr;
  int64_t best_rem = -1;
  for (Lane* ln : {&L, &C})
    for (Live* e : ln->live) {
      const int64_t rem = e->r.iterations - e->done;
      if (rem > best_rem) {
        best_rem = rem;
        best = e;
      }
    }
  if (!best || (L.live.size() == 1 && L.live[0] == best)) return false;
  if (!L.live.empty()) {  // hysteresis: the lead runs faster, so counts cross often
    const int64_t lead_rem = L.live[0]->r.iterations - L.live[0]->done;
    if (best_rem <= lead_rem + lead_rem / 4) return false;
  }
  if (L.inflight || C.inflight) return true;
  for (Live* e : L.live) C.live.push_back(e);
  L.live.clear();
  C.live.erase(std::find(C.live.begin(), C.live.end(), best));
  L.live.push_back(best);
  return false;
}

void complete(gl_server* s, const Live& e, int status, uint64_t res, bool zero, int lane) {
  gl_completion c;
  std::memset(&c, 0, sizeof(c));
  c.id = e.r.id;
  c.p = e.r.p;
  c.N = e.N;
  c.iterations = e.done;
  c.full = e.r.full;
  c.status = status;
  c.is_zero = zero;
  c.is_prime = (e.r.full && e.done == (int64_t)e.r.p - 2 && zero && status == GL_OK) ? 1 : 0;
  c.res64 = res;
  c.max_roundoff = e.maxerr;
  c.arrival_s = e.r.arrival;
  c.admit_s = e.admit;
  c.done_s = s->now();
  c.attempts = e.attempts;
  c.lane = lane;
  c.n_checkpoints = (int)e.checkpoints.size();
  std::lock_guard<std::mutex> lk(s->mu);
  s->checkpoints[e.r.id] = e.checkpoints;
  s->completions.push_back(c);
  s->n_completed++;
  s->cv.notify_all();
}

void fail(gl_server* s, int rc) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->error == GL_OK) s->error = rc;
  s->stop = true;
  s->cv.notify_all();
}

void builder_main(gl_server* s) {
  for (;;) {
    Live* e = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stop || !s->to_build.empty(); });
      if (s->stop && s->to_build.empty()) return;
      e = s->to_build.front();
      s->to_build.pop_front();
    }
    e->build_rc = s->eng.create(s->eng.ctx, e->r.p, e->N, &e->test);
    std::lock_guard<std::mutex> lk(s->mu);
    s->built.push_back(e);
    s->cv.notify_all();
  }
}

// sizes a request and queues it (or completes it with the sizing error)
void arrive(gl_server* s, const Request& r, int attempts, int above) {
  Live* e = new Live();
  e->r = r;
  e->attempts = attempts;
  int rc = s->eng.signal_size(s->eng.ctx, r.p, s->o.max_bits_per_word, above, &e->N);
  if (rc == GL_OK) rc = s->eng.footprint(s->eng.ctx, r.p, e->N, &e->bytes);
  if (rc != GL_OK) {
    e->admit = s->now();
    complete(s, *e, rc, 0, false, lane_of(s, r));
    delete e;
    return;
  }
  if (above) s->queue.push_front(e);  // a restart goes ahead of the queue
  else s->queue.push_back(e);
}

int nlive(const gl_server* s) {
  int n = 0;
  for (int i = 0; i < s->nlanes; ++i) n += (int)s->lanes[i].live.size();
  return n;
}

void admit(gl_server* s) {
  while (!s->queue.empty() && nlive(s) + s->building < s->o.max_active &&
         s->used + s->queue.front()->bytes <= (size_t)s->o.hbm_budget_bytes) {
    Live* e = s->queue.front();
    s->queue.pop_front();
    e->admit = s->now();
    s->used += e->bytes;
    s->building++;
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.peak_bytes = std::max(s->stats.peak_bytes, s->used);
    s->to_build.push_back(e);
    s->cv.notify_all();
  }
  if (!s->queue.empty() && nlive(s) == 0 && s->building == 0 &&
      s->queue.front()->bytes > (size_t)s->o.hbm_budget_bytes) {
    Live* e = s->queue.front();  // can never fit: reject rather than wait forever
    s->queue.pop_front();
    e->admit = s->now();
    complete(s, *e, GL_ERR_NOMEM, 0, false, lane_of(s, e->r));
    delete e;
  }
}

// built tests join their lanes; a failed build completes the request
void collect(gl_server* s) {
  std::vector<Live*> done;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    done.swap(s->built);
  }
  for (Live* e : done) {
    s->building--;
    if (e->build_rc != GL_OK) {
      s->used -= e->bytes;
      complete(s, *e, e->build_rc, 0, false, lane_of(s, e->r));
      delete e;
      continue;
    }
    s->lanes[lane_of(s, e->r)].live.push_back(e);
  }
}

void retire(gl_server* s, int lane, Live* e, int status) {
  uint64_t res = 0;
  int zero = 0;
  if (status == GL_OK) {
    const int rc = s->eng.res64(s->eng.ctx, e->test, &res, &zero);
    if (rc != GL_OK) status = rc;
  }
  s->eng.destroy(s->eng.ctx, e->test);
  e->test = nullptr;
  s->used -= e->bytes;
  if (status == GL_ERR_ROUNDOFF && e->attempts <= s->o.retries) {
    arrive(s, e->r, e->attempts + 1, e->N);  // from S0 = 4 at the next larger length
    delete e;
    return;
  }
  complete(s, *e, status, res, zero != 0, lane);
  delete e;
}

int land(gl_server* s, int li) {
  Lane& ln = s->lanes[li];
  const int64_t k = ln.inflight;
  const int n = (int)ln.members.size();
  std::vector<double> err((size_t)n);
  std::vector<int> st((size_t)n);
  int rc = s->eng.finish(s->eng.ctx, ln.batch, n, err.data(), st.data());
  if (rc != GL_OK) return rc;
  const double dt = std::chrono::duration<double>(Clock::now() - ln.t_start).count();
  ln.busy_s += dt;
  ln.iter_ms = dt * 1e3 / (double)k;
  ln.inflight = 0;
  std::vector<std::pair<Live*, int>> gone;
  double flop = 0.0;
  for (int i = 0; i < n; ++i) {
    Live* e = ln.members[(size_t)i];
    e->done += k;
    e->maxerr = std::max(e->maxerr, err[(size_t)i]);
    flop += flop_alg(e->N) * (double)k;
    if (st[(size_t)i] != GL_OK) {
      gone.push_back({e, st[(size_t)i]});
    } else if (e->done >= e->r.iterations) {
      gone.push_back({e, GL_OK});
    } else if (e->r.full && s->o.checkpoint_every > 0 && e->done % s->o.checkpoint_every == 0) {
      uint64_t r = 0;
      int z = 0;
      rc = s->eng.res64(s->eng.ctx, e->test, &r, &z);
      if (rc != GL_OK) return rc;
      e->checkpoints.push_back({e->done, r});
    }
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.flop_alg += flop;
  }
  if (!gone.empty()) {
    s->eng.close_batch(s->eng.ctx, ln.batch);
    ln.batch = nullptr;
    ln.members.clear();
    for (auto& g : gone) {
      ln.live.erase(std::find(ln.live.begin(), ln.live.end(), g.first));
      retire(s, li, g.first, g.second);
    }
  }
  return GL_OK;
}

int launch(gl_server* s, int li) {
  Lane& ln = s->lanes[li];
  if (ln.members != ln.live) {
    if (ln.batch) s->eng.close_batch(s->eng.ctx, ln.batch);
    ln.batch = nullptr;
    std::vector<void*> tests;
    for (Live* e : ln.live) tests.push_back(e->test);
    const int rc = s->eng.batch(s->eng.ctx, tests.data(), (int)tests.size(), ln.level, &ln.batch);
    if (rc != GL_OK) return rc;
    ln.members = ln.live;
    ln.iter_ms = 0.0;
    ln.rebuilds++;
  }
  ln.peak_live = std::max(ln.peak_live, (int)ln.live.size());
  int64_t k = INT64_MAX;
  for (Live* e : ln.live) {
    k = std::min(k, e->r.iterations - e->done);
    if (e->r.full && s->o.checkpoint_every > 0)
      k = std::min(k, s->o.checkpoint_every - e->done % s->o.checkpoint_every);
  }
  k = std::min<int64_t>(k, ln.iter_ms > 0.0 ? std::max<int64_t>(1, (int64_t)(s->o.step_ms / ln.iter_ms)) : 8);
  ln.t_start = Clock::now();
  const int rc = s->eng.start(s->eng.ctx, ln.batch, k);
  if (rc != GL_OK) return rc;
  ln.inflight = k;
  ln.steps++;
  return GL_OK;
}

void publish_stats(gl_server* s) {
  std::lock_guard<std::mutex> lk(s->mu);
  s->stats.wall_s = s->now();
  for (int i = 0; i < 3; ++i) {
    s->stats.lane_busy_s[i] = s->lanes[i].busy_s;
    s->stats.steps[i] = s->lanes[i].steps;
    s->stats.rebuilds[i] = s->lanes[i].rebuilds;
    s->stats.peak_live[i] = s->lanes[i].peak_live;
  }
  s->stats.live = nlive(s);
  s->stats.queued = (int)s->queue.size();
  s->stats.building = s->building;
  s->stats.bytes_in_use = s->used;
  s->stats.submitted = s->n_submitted;
  s->stats.completed = s->n_completed;
}

void loop_main(gl_server* s) {
  if (s->eng.create == ge_create) cudaSetDevice(s->o.device);
  for (;;) {
    std::deque<Request> fresh;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) break;
      fresh.swap(s->submitted);
    }
    for (const Request& r : fresh) arrive(s, r, 1, 0);
    admit(s);
    collect(s);
    bool busy = false;
    for (int i = 0; i < s->nlanes; ++i) busy = busy || s->lanes[i].inflight > 0;
    if (nlive(s) == 0 && !busy) {
      publish_stats(s);
      std::unique_lock<std::mutex> lk(s->mu);
      // nothing on the GPU: wait for a submission or a finished build
      s->cv.wait_for(lk, std::chrono::milliseconds(20),
                     [&] { return s->stop || !s->submitted.empty() || !s->built.empty(); });
      continue;
    }
    bool progressed = false;
    int rc = GL_OK;
    for (int i = 0; i < s->nlanes && rc == GL_OK; ++i) {
      Lane& ln = s->lanes[i];
      if (ln.inflight) {
        const int r = s->eng.ready(s->eng.ctx, ln.batch);
        if (r < 0) rc = r;
        else if (r == 1) {
          rc = land(s, i);
          progressed = true;
        }
      }
    }
    // a pending move between the lead and chain lanes holds both until they are idle
    const bool hold = rc == GL_OK && promote(s);
    for (int i = 0; i < s->nlanes && rc == GL_OK; ++i) {
      Lane& ln = s->lanes[i];
      if (hold && i < 2) continue;
      if (!ln.live.empty() && !ln.inflight) {
        rc = launch(s, i);
        progressed = true;
      }
    }
    if (rc != GL_OK) {
      fail(s, rc);
      break;
    }
    publish_stats(s);
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(100));
  }
  // stopping: wait for steps in flight, then free every test
  for (int i = 0; i < s->nlanes; ++i) {
    Lane& ln = s->lanes[i];
    if (ln.batch) {
      if (ln.inflight) {
        std::vector<double> err(ln.members.size());
        std::vector<int> st(ln.members.size());
        s->eng.finish(s->eng.ctx, ln.batch, (int)ln.members.size(), err.data(), st.data());
      }
      s->eng.close_batch(s->eng.ctx, ln.batch);
      ln.batch = nullptr;
    }
    for (Live* e : ln.live) {
      s->eng.destroy(s->eng.ctx, e->test);
      delete e;
    }
    ln.live.clear();
  }
  for (Live* e : s->queue) delete e;
  s->queue.clear();
  publish_stats(s);
}

}  // namespace

extern "C" {

int gl_server_default_opts(gl_server_opts* o) {
  if (!o) return GL_ERR_ARG;
  std::memset(o, 0, sizeof(*o));
  o->device = 0;
  o->hbm_budget_bytes = 150e9;
  o->max_active = 512;
  o->step_ms = 50.0;
  o->checkpoint_every = 100000;
  o->max_bits_per_word = 0.0;
  o->retries = 2;
  o->chain_iterations = 100000;
  o->lanes = 3;
  o->build_threads = 2;
  o->error_limit = 0.4;
  o->check_every = 1000;
  return GL_OK;
}

int gl_server_create(const gl_server_opts* opts, const gl_server_engine* engine, gl_server** out) {
  if (!out) return GL_ERR_ARG;
  *out = nullptr;
  gl_server_opts o;
  if (opts) o = *opts;
  else gl_server_default_opts(&o);
  if (o.max_active < 1 || !(o.step_ms > 0.0) || o.build_threads < 1 || o.retries < 0 ||
      !(o.error_limit > 0.0 && o.error_limit <= 0.5) || o.check_every < 1 || o.checkpoint_every < 0 ||
      !(o.hbm_budget_bytes > 0.0))
    return GL_ERR_ARG;
  gl_server* s = new gl_server();
  s->o = o;
  s->nlanes = o.lanes >= 3 ? 3 : (o.lanes == 2 ? 2 : 1);
  if (s->nlanes == 3) {
    s->lanes[0].level = 1;  // lead: the device's highest priority
    s->lanes[1].level = 2;  // chain: between
  } else if (s->nlanes == 2) {
    s->lanes[0].level = 1;
  }
  if (engine) {
    s->eng = *engine;
    if (!s->eng.signal_size || !s->eng.footprint || !s->eng.create || !s->eng.destroy || !s->eng.batch ||
        !s->eng.close_batch || !s->eng.start || !s->eng.ready || !s->eng.finish || !s->eng.res64) {
      delete s;
      return GL_ERR_ARG;
    }
  } else {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || o.device < 0 || o.device >= ndev) {
      delete s;
      return GL_ERR_NODEVICE;
    }
    s->gpu.device = o.device;
    s->gpu.error_limit = o.error_limit;
    s->gpu.check_every = o.check_every;
    s->eng = gl_server_engine{&s->gpu, ge_signal_size, ge_footprint, ge_create, ge_destroy, ge_batch,
                              ge_close_batch, ge_start, ge_ready, ge_finish, ge_res64};
  }
  s->t0 = Clock::now();
  for (int i = 0; i < o.build_threads; ++i) s->builders.emplace_back(builder_main, s);
  s->loop_thread = std::thread(loop_main, s);
  *out = s;
  return GL_OK;
}

int gl_server_submit(gl_server* s, int64_t id, int p, int64_t iterations) {
  if (!s || p < 3 || iterations < 0) return GL_ERR_ARG;
  Request r;
  r.id = id;
  r.p = p;
  r.full = iterations == 0;
  r.iterations = r.full ? (int64_t)p - 2 : iterations;
  r.arrival = s->now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return s->error != GL_OK ? s->error : GL_ERR_STATE;
  s->submitted.push_back(r);
  s->n_submitted++;
  s->cv.notify_all();
  return GL_OK;
}

int gl_server_poll(gl_server* s, gl_completion* out, int max, int* n, double timeout_ms) {
  if (!s || !n || max < 0 || (max > 0 && !out)) return GL_ERR_ARG;
  *n = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (timeout_ms > 0.0 && s->completions.empty())
    s->cv.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms),
                   [&] { return s->stop || !s->completions.empty(); });
  while (*n < max && !s->completions.empty()) {
    out[(*n)++] = s->completions.front();
    s->completions.pop_front();
  }
  return s->error;
}

int gl_server_drain(gl_server* s) {
  if (!s) return GL_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv.wait(lk, [&] { return s->stop || s->n_completed >= s->n_submitted; });
  return s->error;
}

int gl_server_checkpoints(gl_server* s, int64_t id, int64_t* iterations, uint64_t* res64, int max, int* n) {
  if (!s || !n || max < 0) return GL_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->checkpoints.find(id);
  if (it == s->checkpoints.end()) return GL_ERR_ARG;
  *n = 0;
  for (const auto& c : it->second) {
    if (*n >= max) break;
    if (iterations) iterations[*n] = c.first;
    if (res64) res64[*n] = c.second;
    (*n)++;
  }
  return GL_OK;
}

int gl_server_get_stats(gl_server* s, gl_server_stats* st) {
  if (!s || !st) return GL_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  *st = s->stats;
  return GL_OK;
}

int gl_server_destroy(gl_server* s) {
  if (!s) return GL_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->loop_thread.joinable()) s->loop_thread.join();
  for (auto& t : s->builders)
    if (t.joinable()) t.join();
  // builds that finished after the loop stopped
  for (Live* e : s->built) {
    if (e->test) s->eng.destroy(s->eng.ctx, e->test);
    delete e;
  }
  for (Live* e : s->to_build) delete e;
  const int err = s->error;
  delete s;
  return err;
}

}  // extern "C"
