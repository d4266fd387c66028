// gl_cli.cpp -- the `gpulucas` executable: the reference's command line over the C ABI.
//
//   gpulucas [-h] [-v] [-q] [-f N] [-n p] [-d dev] [-c freq] [-k iters] [-m fused|plain] [-H h] [-I mode] [p]
//
// Flags follow gpuLucas.cu:374-454: -f FFT length, -n exponent (or positional), -d CUDA
// device, -c checkpoint frequency (iterations) to <p>.chk in the reference's format
// (gpuLucas.cu:1414-1423, 1569-1665); -v verbose, -q quiet.  Added: -k stop after k
// iterations and print Res64, -m execution form, -H column length of the fused layout,
// -I column-pass variant (1 in place, 2 in place + prefetched weights, -1 two buffers).
// Without -f the length is chosen as findSignalSize does (gpuLucas.cu:1064-1187).  A run
// that finds <p>.chk (or <p>.chk.bak) resumes from it.  SIGINT / SIGTERM write a
// checkpoint and exit (gpuLucas.cu:365-369, 1425-1429).  A full test appends the result
// line (gpuLucas.cu:1514-1548) to results.txt and removes its checkpoint files
// (gpuLucas.cu:628-632).  Exit status: 0 done, 1 usage, 2 bad arguments, 3 library error,
// 130 interrupted.
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gpulucas.h"

namespace {

volatile std::sig_atomic_t g_stop = 0;
void on_signal(int) { g_stop = 1; }

void usage() {
  std::fprintf(stderr,
               "usage: gpulucas [-h] [-v] [-q] [-f N] [-n p] [-d dev] [-c freq] [-k iters] [-m fused|plain] "
               "[-H h] [-I mode] [-R radix] [-P mode] [p]\n"
               "  -f N    FFT length (even, N/2 = 2^a 3^b 5^c 7^d); default: timed search\n"
               "  -n p    exponent of 2^p - 1 (or give it as the last argument)\n"
               "  -d dev  CUDA device\n"
               "  -c freq checkpoint every freq iterations to <p>.chk (resumed automatically)\n"
               "  -k k    stop after k iterations and print Res64 (default: full p-2 test)\n"
               "  -m      fused (default) or plain execution form\n"
               "  -H h    fused layout column length\n"
               "  -I mode column passes: 1 in place, 2 in place + prefetch, 3 two columns per CTA,\n"
               "          4 two columns per CTA forward + prefetch inverse, -1 two buffers\n"
               "  -R r    largest radix of the row DFTs (8, 4 or 2)\n"
               "  -P mode row pass: -1 any radix, 1 radices 4/3/2 only, 2 the same with L1 stage values\n"
               "  -v -q   verbose / quiet\n");
}

bool exists(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (f) std::fclose(f);
  return f != nullptr;
}

int fail(const char* what, int st) {
  std::fprintf(stderr, "%s: %s (%d)\n", what, gl_error_string(st), st);
  return 3;
}

}  // namespace

int main(int argc, char** argv) {
  bool verbose = false, quiet = false;
  int N = 0, p = 0, dev = 0, fft_h = 0, mode = GL_MODE_FUSED, inplace = 0, row_radix = 0, row_pass = 0;
  long long freq = 0, k = 0;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&](const char* flag) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value\n", flag);
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-h") {
      usage();
      return 1;
    } else if (a == "-v") verbose = true;
    else if (a == "-q") quiet = true;
    else if (a == "-f") N = std::atoi(next("-f"));
    else if (a == "-n") p = std::atoi(next("-n"));
    else if (a == "-d") dev = std::atoi(next("-d"));
    else if (a == "-c") freq = std::atoll(next("-c"));
    else if (a == "-k") k = std::atoll(next("-k"));
    else if (a == "-H") fft_h = std::atoi(next("-H"));
    else if (a == "-I") inplace = std::atoi(next("-I"));
    else if (a == "-R") row_radix = std::atoi(next("-R"));
    else if (a == "-P") row_pass = std::atoi(next("-P"));
    else if (a == "-m") {
      const std::string m = next("-m");
      if (m == "fused") mode = GL_MODE_FUSED;
      else if (m == "plain") mode = GL_MODE_PLAIN;
      else {
        std::fprintf(stderr, "-m takes fused or plain\n");
        return 2;
      }
    } else if (!a.empty() && a[0] != '-') p = std::atoi(a.c_str());
    else {
      usage();
      return 2;
    }
  }
  if (p <= 0) {
    std::fprintf(stderr, "testPrime not specified, aborting\n");
    return 2;
  }
  if (freq < 0 || k < 0 || N < 0) {
    usage();
    return 2;
  }
  const std::string chk = std::to_string(p) + ".chk";
  long long resume_at = -1;
  if (exists(chk) || exists(chk + ".bak")) {
    int Nc = 0;
    int64_t it = 0;
    const int st = gl_checkpoint_read(chk.c_str(), p, &Nc, &it, nullptr);
    if (st != GL_OK) std::fprintf(stderr, "ignoring checkpoint: %s\n", gl_error_string(st));
    else if (N && N != Nc) std::fprintf(stderr, "checkpoint %s has N = %d, not %d; not resuming\n", chk.c_str(), Nc, N);
    else {
      N = Nc;
      resume_at = it;
    }
  }
  gl_plan_opts o;
  gl_default_opts(&o);
  o.device = dev;
  o.mode = mode;
  o.fft_h = fft_h;
  o.col_inplace = inplace;
  o.max_radix_row = row_radix;
  o.row_pass = row_pass;
  if (!N) {
    double ms = 0.0, err = 0.0;
    const int st = gl_find_signal_size(p, &o, &N, &ms, &err);
    if (st != GL_OK) return fail("findSignalSize", st);
    if (!quiet) std::printf("Optimal signalSize detected: %d (%.4f ms/iter, trial round-off %.4f)\n", N, ms, err);
  }
  const long long total = k ? k : (long long)p - 2;
  std::signal(SIGINT, on_signal);
  std::signal(SIGTERM, on_signal);
  gl_plan* pl = nullptr;
  int st = gl_plan_create(p, N, &o, &pl);
  if (st != GL_OK) return fail("plan", st);
  gl_plan_info info;
  gl_plan_get_info(pl, &info);
  long long done = 0;
  if (resume_at >= 0) {
    st = gl_plan_resume(pl, chk.c_str());
    if (st != GL_OK) {
      gl_plan_destroy(pl);
      return fail("resume", st);
    }
    done = resume_at;
    if (!quiet) std::printf("Resuming M%d at iteration %lld from %s\n", p, done, chk.c_str());
  }
  if (!quiet)
    std::printf("Testing M%d, word sizes (%d, %d), FFT length %d (%d x %d complex), carry depth %d, form %s\n", p,
                info.lo_bits, info.hi_bits, N, info.fft_h, info.fft_w, info.carry_depth,
                mode == GL_MODE_FUSED ? "fused" : "plain");
  const long long step = freq > 0 ? freq : (total - done > 0 ? total - done : 1);
  double ms_total = 0.0, maxerr = 0.0;
  const long long start = done;
  while (done < total && !g_stop) {
    const long long n = step < total - done ? step : total - done;
    gl_iter_report rep;
    st = gl_iterate(pl, n, &rep);
    if (st != GL_OK) {
      gl_plan_destroy(pl);
      return fail("iterate", st);  // round-off over the limit aborts the test
    }
    done += n;
    ms_total += rep.ms;
    if (rep.max_roundoff > maxerr) maxerr = rep.max_roundoff;
    if (freq > 0 && (done < total || g_stop)) {
      st = gl_checkpoint_write(pl, chk.c_str());
      if (st != GL_OK) std::fprintf(stderr, "checkpoint: %s\n", gl_error_string(st));
      if (verbose) {
        uint64_t r = 0;
        int z = 0;
        gl_get_residue(pl, nullptr, &r, &z);
        std::printf("[%4.1f%%] Iter %lld: %.4f ms/iter, 0x%016llx\n", 100.0 * done / total, done, rep.ms / n,
                    (unsigned long long)r);
      }
    }
  }
  if (g_stop && done < total) {
    gl_checkpoint_write(pl, chk.c_str());
    std::printf("Interrupted at iteration %lld; checkpoint written to %s\n", done, chk.c_str());
    gl_plan_destroy(pl);
    return 130;
  }
  uint64_t res = 0;
  int zero = 0;
  st = gl_get_residue(pl, nullptr, &res, &zero);
  gl_plan_destroy(pl);
  if (st != GL_OK) return fail("residue", st);
  if (k) {
    std::printf("M( %d ) Iter %lld: 0x%016llx, max round-off %.4f, %.4f ms/iter, n = %d\n", p, done,
                (unsigned long long)res, maxerr, ms_total / (double)(done - start > 0 ? done - start : 1), N);
    return 0;
  }
  char line[160];
  if (zero) std::snprintf(line, sizeof line, "M( %d )P, n = %d, gpulucas_gb300", p, N);
  else std::snprintf(line, sizeof line, "M( %d )C, 0x%016llx, n = %d, gpulucas_gb300", p, (unsigned long long)res, N);
  std::printf("%s\n", line);
  if (verbose) std::printf("max round-off %.4f\n", maxerr);
  FILE* f = std::fopen("results.txt", "a");
  if (f) {
    std::fprintf(f, "%s\n", line);
    std::fclose(f);
  }
  std::remove(chk.c_str());
  std::remove((chk + ".bak").c_str());
  return 0;
}
