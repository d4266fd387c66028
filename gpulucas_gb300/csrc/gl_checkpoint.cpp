// gl_checkpoint.cpp -- checkpoints in the reference's <p>.chk format
// (writeCheckpoint / readCheckpoint, gpuLucas.cu:1569-1665).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpulucas.h"
#include "gl_tables.h"

namespace {

constexpr char kName[16] = "gpuLucas";
constexpr char kVersion[16] = "0.9.4";

struct Header {
  char name[16];
  char version[16];
  int p, N, iter;
};

// weights A[j] = 2^(ceil(jp/N) - jp/N) as the reference's d_signal uses them
std::vector<double> weights(int p, int N) {
  std::vector<double> A, Ainv;
  gl::weight_tables(p, N, (double)N, A, Ainv);
  return A;
}

int read_file(const std::string& path, int p, int* N_out, int64_t* iters, int32_t* digits) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return GL_ERR_IO;
  Header h;
  if (std::fread(h.name, 1, 16, f) != 16 || std::fread(h.version, 1, 16, f) != 16 ||
      std::fread(&h.p, sizeof(int), 1, f) != 1 || std::fread(&h.N, sizeof(int), 1, f) != 1 ||
      std::fread(&h.iter, sizeof(int), 1, f) != 1) {
    std::fclose(f);
    return GL_ERR_CHECKPOINT;
  }
  h.name[15] = 0;
  if (std::strcmp(h.name, kName) != 0 || h.p != p || h.N < 16 || (h.N & 1) || h.N > p || h.iter < 1) {
    std::fclose(f);
    return GL_ERR_CHECKPOINT;
  }
  std::vector<double> d((size_t)h.N);
  const size_t got = std::fread(d.data(), sizeof(double), (size_t)h.N, f);
  std::fclose(f);
  if (got != (size_t)h.N) return GL_ERR_CHECKPOINT;
  if (digits) {
    const std::vector<double> A = weights(p, h.N);
    for (int j = 0; j < h.N; ++j) {
      const double v = std::nearbyint(d[j] / A[j]);
      if (!(std::fabs(v) < 2147483647.0) || std::fabs(d[j] / A[j] - v) > 0.25) return GL_ERR_CHECKPOINT;
      digits[j] = (int32_t)v;
    }
  }
  *N_out = h.N;
  *iters = (int64_t)h.iter - 1;
  return GL_OK;
}

}  // namespace

extern "C" {

int gl_checkpoint_read(const char* path, int p, int* N_out, int64_t* iterations_out, int32_t* digits_out) {
  if (!path || !N_out || !iterations_out || p < 3) return GL_ERR_ARG;
  int rc = read_file(path, p, N_out, iterations_out, digits_out);
  if (rc != GL_OK) {
    const int rc2 = read_file(std::string(path) + ".bak", p, N_out, iterations_out, digits_out);
    if (rc2 == GL_OK) return GL_OK;
  }
  return rc;
}

int gl_checkpoint_write(gl_plan* plan, const char* path) {
  if (!plan || !path) return GL_ERR_ARG;
  gl_plan_info info;
  int rc = gl_plan_get_info(plan, &info);
  if (rc != GL_OK) return rc;
  const int N = info.N, p = info.p;
  std::vector<int32_t> digit((size_t)N);
  std::vector<int8_t> hi((size_t)N);
  if ((rc = gl_get_carry_state(plan, digit.data(), hi.data())) != GL_OK) return rc;
  gl_iter_report rep{};
  if ((rc = gl_sync_status(plan, &rep)) != GL_OK && rc != GL_ERR_ROUNDOFF) return rc;
  const std::vector<double> A = weights(p, N);
  std::vector<double> d((size_t)N);
  for (int j = 0; j < N; ++j) d[j] = A[j] * (double)(digit[j] + hi[j == 0 ? N - 1 : j - 1]);
  Header h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.name, kName, sizeof(kName));
  std::memcpy(h.version, kVersion, sizeof(kVersion));
  h.p = p;
  h.N = N;
  h.iter = (int)(rep.total_iterations + 1);
  const std::string tmp = std::string(path) + ".tmp", bak = std::string(path) + ".bak";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return GL_ERR_IO;
  bool ok = std::fwrite(h.name, 1, 16, f) == 16 && std::fwrite(h.version, 1, 16, f) == 16 &&
            std::fwrite(&h.p, sizeof(int), 1, f) == 1 && std::fwrite(&h.N, sizeof(int), 1, f) == 1 &&
            std::fwrite(&h.iter, sizeof(int), 1, f) == 1 &&
            std::fwrite(d.data(), sizeof(double), (size_t)N, f) == (size_t)N;
  ok = (std::fflush(f) == 0) && ok;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    std::remove(tmp.c_str());
    return GL_ERR_IO;
  }
  std::remove(bak.c_str());
  std::rename(path, bak.c_str());  // no previous checkpoint is fine
  if (std::rename(tmp.c_str(), path) != 0) return GL_ERR_IO;
  return GL_OK;
}

int gl_plan_resume(gl_plan* plan, const char* path) {
  if (!plan || !path) return GL_ERR_ARG;
  gl_plan_info info;
  int rc = gl_plan_get_info(plan, &info);
  if (rc != GL_OK) return rc;
  int N = 0;
  int64_t k = 0;
  std::vector<int32_t> digits((size_t)info.N);
  int32_t* dst = digits.data();
  // the header's N must match the plan before the body is decoded
  if ((rc = gl_checkpoint_read(path, info.p, &N, &k, nullptr)) != GL_OK) return rc;
  if (N != info.N) return GL_ERR_CHECKPOINT;
  if ((rc = gl_checkpoint_read(path, info.p, &N, &k, dst)) != GL_OK) return rc;
  std::vector<int8_t> hi((size_t)N, 0);
  return gl_set_carry_state(plan, dst, hi.data(), k);
}

}  // extern "C"
