// gl_noalloc.cu -- Lucas-Lehmer iterations for callers that cannot allocate device
// memory.
//
// Some callers may not call cudaMalloc at all: code that runs inside a framework
// whose memory pool owns every device allocation, code that must not grow its
// footprint once a service is running, or code whose allocation calls would
// synchronise a device it shares with latency-sensitive work.  gl_iterate_noalloc
// serves them: the caller passes device buffers for the input and output products,
// and everything else the iterations need -- the two FFT work arrays, the weight,
// flag and twiddle tables of the test, the carry-save digits and the round-off
// status word -- lives in one file-scope __device__ array below.  It is sized for
// N <= kNoAllocMaxN (65536 words, about 3.3 MiB) and stays resident on every GPU that
// loads this library until the process exits.
//
// The iterations are the plain form (one kernel per reference step), launched
// through the same launchers as a plan of GL_MODE_PLAIN, so the products equal those
// of gl_iterate bit for bit.
#include <cstring>
#include <mutex>

#include "gl_internal.h"
#include "gl_tables.h"

namespace gl {
namespace {

constexpr int kNoAllocMaxN = 65536;
constexpr int kNoAllocMaxM = kNoAllocMaxN / 2;
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
// byte offsets of the sub-buffers inside the scratch array
constexpr size_t kOffZ = 0;
constexpr size_t kOffZ2 = kOffZ + align256(sizeof(DevCplx) * kNoAllocMaxM);
constexpr size_t kOffTwM = kOffZ2 + align256(sizeof(DevCplx) * kNoAllocMaxM);
constexpr size_t kOffPair = kOffTwM + align256(sizeof(DevCplx) * kNoAllocMaxM);
constexpr size_t kOffA = kOffPair + align256(sizeof(DevCplx) * kNoAllocMaxM);
constexpr size_t kOffAinv = kOffA + align256(sizeof(double) * kNoAllocMaxN);
constexpr size_t kOffDigit = kOffAinv + align256(sizeof(double) * kNoAllocMaxN);
constexpr size_t kOffHi = kOffDigit + align256(sizeof(int) * kNoAllocMaxN);
constexpr size_t kOffFlags = kOffHi + align256(kNoAllocMaxN);
constexpr size_t kOffStatus = kOffFlags + align256(kNoAllocMaxN);
constexpr size_t kScratchBytes = kOffStatus + align256(sizeof(Status));

// The scratch.  In host code this name is only a host-side stand-in for the symbol,
// never a device address: the address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Host staging for the per-test tables, reused by every call (no host allocation).
static DevCplx h_twM[kNoAllocMaxM];
static DevCplx h_pair[kNoAllocMaxM];
static double h_A[kNoAllocMaxN];
static double h_Ainv[kNoAllocMaxN];
static unsigned char h_flags[kNoAllocMaxN];
static Status h_status;

struct DeviceSlot {
  unsigned char* base = nullptr;  // device address of g_noalloc_scratch on this device
  int p = 0, N = 0;               // test whose tables the scratch holds
};
static DeviceSlot g_slots[kMaxDevices];
static std::mutex g_mutex;  // host-side state: staging buffers and the slots

// Fill the host staging tables for (p, N) with the entry helpers a GL_MODE_PLAIN plan's
// tables are built from (gl_tables.cpp), so the two cannot drift apart.
void build_tables(int p, int N) {
  const int M = N / 2;
  for (int k = 0; k < M; ++k) {
    const HostCplx w = twiddle(k, M);
    const HostCplx c = pair_coeff(k, M);
    h_twM[k] = {w.re, w.im};
    h_pair[k] = {c.re, c.im};
  }
  for (int j = 0; j < N; ++j) weight_entry(p, N, j, (double)M, &h_A[j], &h_Ainv[j]);
  for (int j = 0; j < N; ++j) h_flags[j] = word_flags(p, N, j);
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int gl_iterate_noalloc(int p, int N, const int64_t* ll_in, int64_t* ll_out, int64_t iters,
                                  double* max_roundoff, void* stream) {
  if (!ll_in || !ll_out || iters < 0) return GL_ERR_ARG;
  if (p < 3 || N < 16 || (N & 1) || N > p) return GL_ERR_ARG;
  if (N > kNoAllocMaxN) return GL_ERR_TOO_LARGE;
  {
    // the same buffer is fine; buffers that share only part of their words are not
    const int64_t* out_c = ll_out;
    if (out_c != ll_in && out_c < ll_in + N && ll_in < out_c + N) return GL_ERR_ARG;
  }
  const int n = slice_depth(p, N);
  if (n < 0) return GL_ERR_RATIO;
  const int M = N / 2;
  PlainGeom pg{};
  // radices of the plain form (<= 4), by the helper a GL_MODE_PLAIN plan uses
  pg.nst = radix_plan_into(M, 4, pg.radix, 40);
  if (pg.nst <= 0) return GL_ERR_SIZE;
  pg.threads = 256;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  {
    // the call waits for its stream, which a stream being captured into a graph cannot do
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
      cudaGetLastError();
      return GL_ERR_CUDA;
    }
    if (cs != cudaStreamCaptureStatusNone) return GL_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GL_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GL_ERR_ARG;

  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceSlot& slot = g_slots[dev];
  {
    // The array's device address, looked up with this device current on every call (the
    // lookup allocates nothing).  If it moved -- the context was reset and the module
    // loaded again -- the tables the slot remembers are gone too.
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return GL_ERR_CUDA;
    if (static_cast<unsigned char*>(ptr) != slot.base) {
      slot.base = static_cast<unsigned char*>(ptr);
      slot.p = slot.N = 0;
    }
  }
  unsigned char* base = slot.base;
  if (slot.p != p || slot.N != N) {
    build_tables(p, N);
    if (cudaMemcpyAsync(base + kOffTwM, h_twM, sizeof(DevCplx) * M, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(base + kOffPair, h_pair, sizeof(DevCplx) * M, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(base + kOffA, h_A, sizeof(double) * N, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(base + kOffAinv, h_Ainv, sizeof(double) * N, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(base + kOffFlags, h_flags, N, cudaMemcpyHostToDevice, s)) {
      slot.p = slot.N = 0;
      return GL_ERR_CUDA;
    }
    slot.p = p;
    slot.N = N;
  }

  IterArgs a{};
  a.N = N; a.M = M; a.LO = p / N; a.n = n;
  a.ll = reinterpret_cast<long long*>(ll_out);
  a.flags = base + kOffFlags;
  a.A = reinterpret_cast<const double*>(base + kOffA);
  a.Ainv = reinterpret_cast<const double*>(base + kOffAinv);
  a.Z = reinterpret_cast<DevCplx*>(base + kOffZ);
  a.Z2 = reinterpret_cast<DevCplx*>(base + kOffZ2);
  a.twM = reinterpret_cast<const DevCplx*>(base + kOffTwM);
  a.twPair = reinterpret_cast<const DevCplx*>(base + kOffPair);
  a.digit = reinterpret_cast<int*>(base + kOffDigit);
  a.hi = reinterpret_cast<signed char*>(base + kOffHi);
  a.status = reinterpret_cast<Status*>(base + kOffStatus);

  // the status word keeps the previous call's contents: clear it
  if (cudaMemsetAsync(a.status, 0, sizeof(Status), s) != cudaSuccess) return GL_ERR_CUDA;
  if (ll_out != ll_in &&
      cudaMemcpyAsync(ll_out, ll_in, sizeof(int64_t) * N, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return GL_ERR_CUDA;
  if (launch_dice(a, s) != cudaSuccess) return GL_ERR_CUDA;
  for (int64_t i = 0; i < iters; ++i)
    if (launch_plain_iteration(a, pg, s) != cudaSuccess) return GL_ERR_CUDA;
  if (cudaMemcpyAsync(&h_status, a.status, sizeof(Status), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GL_ERR_CUDA;
  const double e = (double)h_status.maxerr64 * 0x1p-64;
  if (max_roundoff) *max_roundoff = e;
  if (h_status.flags) return GL_ERR_OVERFLOW;
  if (e >= 0.4) return GL_ERR_ROUNDOFF;
  return GL_OK;
}
