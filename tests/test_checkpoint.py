"""Checkpoints in the reference's <p>.chk format (gpuLucas.cu:1569-1665).

Files are made the way writeCheckpoint does (char[16] "gpuLucas", char[16] "0.9.4",
int p, int N, int iter, N doubles of d_signal = A[j] (digit[j] + hi[j-1])) from the
oracle's state, so these tests pin the format without the reference binary.
"""
import os
import struct

import numpy as np
import pytest


def write_reference_checkpoint(path, p, N, iter_field, d_signal, name=b"gpuLucas", version=b"0.9.4"):
    with open(path, "wb") as f:
        f.write(name.ljust(16, b"\0")[:16])
        f.write(version.ljust(16, b"\0")[:16])
        f.write(struct.pack("<iii", p, N, iter_field))
        f.write(np.asarray(d_signal, np.float64).tobytes())


def oracle_state(orc, p, N, k):
    o = orc.IBDWT(p, N).iterate(k)
    d, h = o.state()
    return o.signal(), d.astype(np.int64) + np.roll(h.astype(np.int64), 1), o


def test_read_reference_format(gl, orc, tmp_path):
    p, N, k = 44497, 2048, 123
    sig, v, _ = oracle_state(orc, p, N, k)
    path = str(tmp_path / f"{p}.chk")
    write_reference_checkpoint(path, p, N, k + 1, sig)   # the reference writes iter = k + 1
    N2, k2, digits = gl.checkpoint_read(path, p)
    assert (N2, k2) == (N, k)
    assert np.array_equal(digits, v)


def test_read_falls_back_to_backup(gl, orc, tmp_path):
    p, N, k = 12379, 640, 50
    sig, v, _ = oracle_state(orc, p, N, k)
    path = str(tmp_path / f"{p}.chk")
    write_reference_checkpoint(path + ".bak", p, N, k + 1, sig)
    N2, k2, digits = gl.checkpoint_read(path, p)
    assert (N2, k2) == (N, k) and np.array_equal(digits, v)


@pytest.mark.parametrize("what", ["name", "p", "truncated", "garbage"])
def test_read_rejects_bad_files(gl, orc, tmp_path, what):
    p, N, k = 12379, 640, 20
    sig, _, _ = oracle_state(orc, p, N, k)
    path = str(tmp_path / f"{p}.chk")
    if what == "name":
        write_reference_checkpoint(path, p, N, k + 1, sig, name=b"otherApp")
    elif what == "p":
        write_reference_checkpoint(path, p + 2, N, k + 1, sig)
    elif what == "truncated":
        write_reference_checkpoint(path, p, N, k + 1, sig[: N // 2])
    else:
        write_reference_checkpoint(path, p, N, k + 1, sig * 1.3 + 0.37)
    with pytest.raises(gl.GLError) as ei:
        gl.checkpoint_read(path, p)
    assert ei.value.status == gl.GL_ERR_CHECKPOINT


def test_read_missing(gl, tmp_path):
    with pytest.raises(gl.GLError) as ei:
        gl.checkpoint_read(str(tmp_path / "nothing.chk"), 12379)
    assert ei.value.status == gl.GL_ERR_IO


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1], ids=["fused", "plain"])
def test_resume_from_reference_checkpoint(gl, orc, tmp_path, mode):
    """A run checkpointed by the reference's algorithm continues here bit for bit."""
    p, N, k, more = 100003, 5184, 777, 250
    sig, _, o = oracle_state(orc, p, N, k)
    path = str(tmp_path / f"{p}.chk")
    write_reference_checkpoint(path, p, N, k + 1, sig)
    with gl.Plan(p, N, mode=mode) as pl:
        pl.resume(path)
        pl.iterate(more)
        o.iterate(more)
        assert np.array_equal(pl.products(), o.ll())
        assert pl.res64() == orc.Exact(p).iterate(k + more).res64()


@pytest.mark.gpu
def test_write_then_resume(gl, orc, tmp_path):
    p, N = 1000003, 54432
    path = str(tmp_path / f"{p}.chk")
    with gl.Plan(p, N) as a:
        a.iterate(300)
        a.checkpoint_write(path)
        a.iterate(100)
        a.checkpoint_write(path)          # the first file becomes path.bak
        a.iterate(150)
        ref = a.products()
    assert os.path.exists(path + ".bak")
    assert gl.checkpoint_read(path + ".bak", p, with_digits=False)[1] == 300
    with gl.Plan(p, N) as b:
        b.resume(path)
        b.iterate(150)
        assert np.array_equal(b.products(), ref)
    o = orc.IBDWT(p, N).iterate(550)
    assert np.array_equal(ref, o.ll())


@pytest.mark.gpu
def test_cli_checkpoint_resume_and_result_line(tmp_path):
    """The CLI with -c writes <p>.chk, a second run resumes from it, a full test appends
    the reference's result line to results.txt and removes the checkpoint files."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, PYTHONPATH=root)
    p, N = 4423, 256
    r1 = subprocess.run([sys.executable, "-m", "gpulucas_gb300", "-f", str(N), "-c", "1000", "-k", "2000", str(p)],
                        cwd=tmp_path, env=env, capture_output=True, text=True, timeout=300)
    assert r1.returncode == 0, r1.stderr
    assert os.path.exists(tmp_path / f"{p}.chk")
    r2 = subprocess.run([sys.executable, "-m", "gpulucas_gb300", "-c", "1000", str(p)],
                        cwd=tmp_path, env=env, capture_output=True, text=True, timeout=300)
    assert r2.returncode == 0, r2.stderr
    assert "Resuming" in r2.stdout
    assert (tmp_path / "results.txt").read_text().strip() == f"M( {p} )P, n = {N}, gpulucas_gb300"
    assert not os.path.exists(tmp_path / f"{p}.chk")


CLI_BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gpulucas_gb300", "gpulucas")


def test_native_cli_usage_and_errors(tmp_path):
    """The C++ `gpulucas` executable: usage, argument errors, and a loud failure (no CPU
    path) when no GPU is usable."""
    import subprocess
    if not os.path.exists(CLI_BIN):
        pytest.skip("gpulucas executable not built")
    r = subprocess.run([CLI_BIN, "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "usage: gpulucas" in r.stderr
    r = subprocess.run([CLI_BIN, "-f", "2048"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "testPrime not specified" in r.stderr
    r = subprocess.run([CLI_BIN, "-m", "fast", "44497"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    r = subprocess.run([CLI_BIN, "-d", "99", "-k", "10", "-f", "2048", "44497"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 3 and not os.path.exists(tmp_path / "results.txt")


@pytest.mark.gpu
def test_native_cli_res64_checkpoint_and_result_line(tmp_path):
    """The C++ executable: Res64 after k iterations equals the golden value; -c writes
    <p>.chk in the reference's format, a second run resumes, a full test appends the
    result line and removes the checkpoint files."""
    import subprocess
    r = subprocess.run([CLI_BIN, "-k", "1000", "-f", "2048", "44497"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Iter 1000: 0xd76d70f8f0325ccb" in r.stdout
    p, N = 4423, 256
    r1 = subprocess.run([CLI_BIN, "-f", str(N), "-c", "1000", "-k", "2000", str(p)], cwd=tmp_path,
                        capture_output=True, text=True, timeout=300)
    assert r1.returncode == 0, r1.stderr
    assert os.path.exists(tmp_path / f"{p}.chk")
    r2 = subprocess.run([CLI_BIN, "-c", "1000", "-m", "plain", str(p)], cwd=tmp_path, capture_output=True, text=True,
                        timeout=300)
    assert r2.returncode == 0, r2.stderr
    assert "Resuming" in r2.stdout
    assert (tmp_path / "results.txt").read_text().strip() == f"M( {p} )P, n = {N}, gpulucas_gb300"
    assert not os.path.exists(tmp_path / f"{p}.chk")
