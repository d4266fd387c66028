"""The recipe that builds the reference gpuLucas program as an oracle (CPU checks).

* The double-double stand-in for QD (oracle/ref_shim/qd/dd_real.h) gives the weights of
  computeWeightVectors (gpuLucas.cu:673-686) equal to mpmath at 140 bits rounded to
  double, on the committed golden samples.
* Every patch of oracle/build_ref.py matches the reference source exactly once (where the
  reference checkout is present) and the staged copy differs from it only there.
* The staged copy compiles for sm_103a and links cuFFT.
"""
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SHIM = os.path.join(ROOT, "oracle", "ref_shim")

# computeWeightVectors (gpuLucas.cu:673-686) evaluated with the shim, for (p, N, j) read
# from standard input; prints A[j] and Ainv[j] as hexadecimal floats.
_WEIGHTS_PROG = r"""
#include <cstdio>
#include <qd/dd_real.h>
int main() {
  int p, N, n;
  while (std::scanf("%d %d %d", &p, &N, &n) == 3) {
    dd_real dd_N = dd_real(N);
    dd_real dd_2 = dd_real(2.0);
    for (int i = 0; i < n; ++i) {
      int j;
      if (std::scanf("%d", &j) != 1) return 1;
      dd_real e = dd_real(j) * dd_real(p) / dd_N;
      dd_real A = pow(dd_2, ceil(e) - e);
      dd_real Ai = (1.0 / A) / dd_N;
      std::printf("%a %a\n", to_double(A), to_double(Ai));
    }
  }
  return 0;
}
"""


def _build_ref_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gl_build_ref_t", os.path.join(ROOT, "oracle", "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_shim_weights_equal_mpmath(tmp_path):
    src = tmp_path / "w.cpp"
    src.write_text(_WEIGHTS_PROG)
    exe = tmp_path / "w"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-I", SHIM, str(src), "-o", str(exe)], check=True)
    with open(os.path.join(HERE, "golden", "weights.json")) as f:
        golden = json.load(f)
    stdin = "".join(f"{e['p']} {e['N']} {len(e['j'])} " + " ".join(map(str, e["j"])) + "\n" for e in golden)
    out = subprocess.run([str(exe)], input=stdin, capture_output=True, text=True, check=True).stdout.split("\n")
    i = 0
    for e in golden:
        for j, a, ai in zip(e["j"], e["A"], e["Ainv"]):
            A, Ai = (float.fromhex(t) for t in out[i].split())
            assert (A, Ai) == (float.fromhex(a), float.fromhex(ai)), (e["p"], e["N"], j)
            i += 1
    assert i > 1000


def test_shim_exp_log_pow():
    """exp, log and pow of the shim within 2^-100 relative of mpmath at 140 bits."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 140
    prog = r"""
#include <cstdio>
#include <qd/dd_real.h>
int main() {
  double xs[] = {0.0, 1e-9, 0.25, 0.5, 0.693, 1.0, 3.7, -2.5, 20.0};
  for (double x : xs) {
    dd_real e = exp(dd_real(x));
    dd_real l = log(dd_real((x < 0 ? -x : x) + 1.5));
    dd_real p = pow(dd_real(2.0), dd_real(x / 8));
    dd_real q = pow(dd_real(3.0), dd_real(x / 8));
    std::printf("%a %a %a %a %a %a %a %a\n", e.x[0], e.x[1], l.x[0], l.x[1], p.x[0], p.x[1], q.x[0], q.x[1]);
  }
  return 0;
}
"""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        with open(src, "w") as f:
            f.write(prog)
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-I", SHIM, src, "-o", os.path.join(d, "t")], check=True)
        lines = subprocess.run([os.path.join(d, "t")], capture_output=True, text=True, check=True).stdout.split("\n")
    xs = [0.0, 1e-9, 0.25, 0.5, 0.693, 1.0, 3.7, -2.5, 20.0]
    for x, line in zip(xs, lines):
        v = [mpmath.mpf(float.fromhex(t)) for t in line.split()]
        got = [v[0] + v[1], v[2] + v[3], v[4] + v[5], v[6] + v[7]]
        want = [mpmath.exp(x), mpmath.log(abs(x) + 1.5), mpmath.power(2, mpmath.mpf(x) / 8),
                mpmath.power(3, mpmath.mpf(x) / 8)]
        for g, w in zip(got, want):
            assert abs(g - w) <= abs(w) * mpmath.mpf(2) ** -100, (x, g, w)


def test_patches_match_reference_once():
    br = _build_ref_module()
    ref = br.reference_dir()
    if not all(os.path.isfile(os.path.join(ref, s)) for s in br.SOURCES):
        pytest.skip("no reference checkout here")
    for fname, lines, old, new, why in br.PATCHES:
        with open(os.path.join(ref, fname), encoding="latin-1") as f:
            text = f.read()
        assert text.count(old) == 1, (fname, lines)
        assert old != new and why


def test_staged_copy_differs_only_at_patches(tmp_path, monkeypatch):
    br = _build_ref_module()
    ref = br.reference_dir()
    if not all(os.path.isfile(os.path.join(ref, s)) for s in br.SOURCES):
        pytest.skip("no reference checkout here")
    monkeypatch.setattr(br, "SRC_DIR", str(tmp_path / "src"))
    assert br.stage(ref)
    import difflib
    changed = 0
    for s in br.SOURCES:
        with open(os.path.join(ref, s), encoding="latin-1") as f:
            a = f.read().splitlines()
        with open(tmp_path / "src" / s, encoding="latin-1") as f:
            b = f.read().splitlines()
        assert len(a) == len(b)
        for line in difflib.unified_diff(a, b, lineterm="", n=0):
            if line.startswith("-") and not line.startswith("---"):
                changed += 1
    assert changed == len(br.PATCHES)
    assert (tmp_path / "src" / "PROVENANCE").read_text().count("patch ") == len(br.PATCHES)


def test_staged_copy_compiles(tmp_path, monkeypatch):
    br = _build_ref_module()
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no nvcc")
    ref = br.reference_dir()
    src_dir = tmp_path / "src"
    monkeypatch.setattr(br, "SRC_DIR", str(src_dir))
    monkeypatch.setattr(br, "BINARY", str(tmp_path / "gpuLucas"))
    if not br.stage(ref):
        staged = os.path.join(ROOT, "oracle", "_ref", "src")
        if not os.path.isdir(staged):
            pytest.skip("neither a reference checkout nor a staged copy")
        shutil.copytree(staged, src_dir)
    out = br.compile_staged()
    assert os.path.isfile(out) and os.access(out, os.X_OK)


# A stand-in for the reference program's reporting protocol (gpuLucas.cu:1399-1478,
# 1641-1665): checkpoint every K iterations with the "Iter k" line, the Res64 with -v,
# one more checkpoint and exit 0 on SIGINT.  The "state" is k * (1, 2, ..., N).
_FAKE_PROG = r'''#!/usr/bin/env python3
import signal, struct, sys, time, os
args = sys.argv[1:]
opts = {}
verbose = False
i = 0
while i < len(args):
    if args[i] in ("-d", "-f", "-c"):
        opts[args[i]] = int(args[i + 1]); i += 2
    elif args[i] == "-v":
        verbose = True; i += 1
    else:
        p = int(args[i]); i += 1
N, K = opts["-f"], opts["-c"]
stop = [False]
signal.signal(signal.SIGINT, lambda *a: stop.__setitem__(0, True))
for t in range(3):
    print(f"[{t}/50]: iteration {t}: max abs error = 0.0{t + 1}0000", flush=True)
def write(it):
    name = f"{p}.chk"
    if os.path.exists(name):
        os.replace(name, name + ".bak")
    with open(name, "wb") as f:
        f.write(b"gpuLucas".ljust(16, b"\0") + b"0.9.4".ljust(16, b"\0"))
        f.write(struct.pack("<iii", p, N, it))
        f.write(struct.pack(f"<{N}d", *[(it - 1) * (j + 1.0) for j in range(N)]))
it = 2
while it < p:
    time.sleep(0.0005)
    if it % K == 1 or stop[0]:
        write(it)
        if stop[0]:
            sys.exit(0)
        tail = f", 0x{(it - 1) * 0x1111:016x}" if verbose else ""
        print(f"[ 0.1%] Iter {it - 1:9d}: {0.25 + it * 1e-6:6.3f} ms/iter, ETA 01:02:03{tail}", flush=True)
    it += 1
'''


def test_runner_protocol_with_fake_program(tmp_path, monkeypatch):
    from oracle import refrun
    fake = tmp_path / "gpuLucas"
    fake.write_text(_FAKE_PROG)
    fake.chmod(0o755)
    monkeypatch.setattr(refrun, "BINARY", str(fake))
    run = refrun.run(100003, 64, every=50, checkpoints=3, verbose=True, capture_state=True, timeout=60)
    assert [k for k, _, _ in run.checkpoints] == [50, 100, 150]
    assert run.res64(100) == 100 * 0x1111
    assert run.trial_maxerr == [0.01, 0.02, 0.03]
    k, sig = run.state
    assert k == 50 and sig.shape == (64,) and (sig == 50.0 * (1 + __import__("numpy").arange(64))).all()
    assert abs(run.ms_per_iter(-1) - (0.25 + 151e-6)) < 1e-3
    assert run.returncode == 0
    quiet = refrun.run(100003, 64, every=20, checkpoints=1, verbose=False, timeout=60)
    assert quiet.checkpoints[0][0] == 20 and quiet.checkpoints[0][2] is None


def test_runner_kills_on_timeout(tmp_path, monkeypatch):
    from oracle import refrun
    fake = tmp_path / "gpuLucas"
    fake.write_text("#!/bin/sh\nexec sleep 30\n")
    fake.chmod(0o755)
    monkeypatch.setattr(refrun, "BINARY", str(fake))
    with pytest.raises(TimeoutError):
        refrun.run(100003, 64, every=50, timeout=1.5)
