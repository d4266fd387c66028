"""include/gpulucas.hpp: the host/device llintToBalInt<n> restatement of the reference's
carry semantics, compiled as plain C++ (no GPU), against the oracle's dicing
(IrrBaseBalanced.cu:52-110) on random products."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "gpulucas.hpp"
int main(int argc, char** argv) {
  int p = atoi(argv[1]), N = atoi(argv[2]), n = atoi(argv[3]);
  std::vector<int64_t> ll(N);
  FILE* f = fopen(argv[4], "rb");
  if (fread(ll.data(), 8, N, f) != (size_t)N) return 3;
  fclose(f);
  std::vector<int32_t> d(N);
  std::vector<int8_t> h(N);
  if (gpulucas::llintToBalInt(n, ll.data(), p, N, d.data(), h.data()) != GL_OK) return 4;
  f = fopen(argv[5], "wb");
  fwrite(d.data(), 4, N, f);
  fwrite(h.data(), 1, N, f);
  for (int j = 0; j < N; ++j) { int b = gpulucas::word_bits(p, N, j); fwrite(&b, 4, 1, f); }
  fclose(f);
  return 0;
}
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("hpp")
    src = d / "dice.cpp"
    src.write_text(PROG)
    exe = d / "dice"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("p,N", [(44497, 2048), (100003, 5184), (2976221, 163840), (1000003, 54432)])
def test_llintToBalInt_matches_oracle(prog, tmp_path, orc, gl, p, N):
    n = gl.setSliceAndDice(p, N)
    rng = np.random.default_rng(p)
    ll = rng.integers(-(2 ** 46), 2 ** 46, N, dtype=np.int64)
    ll[:3] = [2 ** 62 - 1, -(2 ** 62), 0]
    fin, fout = tmp_path / "ll.bin", tmp_path / "out.bin"
    ll.tofile(fin)
    subprocess.run([str(prog), str(p), str(N), str(n), str(fin), str(fout)], check=True)
    raw = fout.read_bytes()
    d = np.frombuffer(raw[:4 * N], np.int32)
    h = np.frombuffer(raw[4 * N:5 * N], np.int8)
    bits = np.frombuffer(raw[5 * N:], np.int32)
    d2, h2 = orc.dice(p, N, ll)
    assert (d == d2).all() and (h == h2).all()
    assert (bits == orc.bits(p, N)[0]).all()
