"""Run the reference gpuLucas program (built by ``oracle/build_ref.py``) and read what it
reports: Res64 and ms/iteration at its checkpoints, and the checkpointed FFT input.

TEST INFRASTRUCTURE ONLY (the GPU tests and bench.py's reference-build baseline leg).

How the reference reports (gpuLucas.cu, the reference project):

* ``gpuLucas -f N -c K [-v] p`` first runs ``errorTrial`` (clamp(p/10000, 100, 2500)
  iterations, gpuLucas.cu:529-555), then the main loop from iteration 2
  (gpuLucas.cu:1368-1399).  When ``iter % K == 1`` it writes the checkpoint ``<p>.chk``
  (the previous one becomes ``<p>.chk.bak``) and prints
  ``[pct%] Iter k: x ms/iter, ETA ...`` with k = iter - 1 = the number of squarings done
  from S0 = 4, and with ``-v`` the Res64 of that state after ``, `` (gpuLucas.cu:1414-1478).
  x is the wall time since the previous checkpoint line over the iterations in between
  (cudaEvents, gpuLucas.cu:1432-1444), one checkpoint write included.
* The checkpoint holds a 16-byte name, a 16-byte version, int p, int N, int iter, then the
  N doubles of the weighted signal A[j] (digit[j] + hi[j-1]) -- the next FFT's input
  (gpuLucas.cu:1641-1665).
* SIGINT makes it write one more checkpoint at the next iteration and exit 0
  (gpuLucas.cu:365-369, 598-606, 1414-1429).

The runner works in a scratch directory (the program writes ``<p>.chk`` files into its
working directory and resumes from them, gpuLucas.cu:497-500), stops the process with
SIGSTOP while it reads a checkpoint (so a later checkpoint cannot rotate it away), and
ends the run with SIGINT.  A run that overstays its time limit is killed by its own PID.
"""
from __future__ import annotations

import os
import queue
import re
import shutil
import signal
import subprocess
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BINARY = os.path.join(HERE, "_ref", "gpuLucas")

_CP_LINE = re.compile(r"\]\s*Iter\s+(\d+):\s+([0-9.]+) ms/iter, ETA [^,\n]*(?:, 0x([0-9a-fA-F]+))?")
_ERR_LINE = re.compile(r"max abs error = ([0-9.]+)")


def available() -> bool:
    return os.path.isfile(BINARY) and os.access(BINARY, os.X_OK)


def read_checkpoint(path: str):
    """(p, N, iter, signal) of a reference-format checkpoint file."""
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 44:
        raise ValueError(f"{path}: short checkpoint")
    p, N, it = np.frombuffer(raw[32:44], "<i4")
    need = 44 + 8 * int(N)
    if len(raw) < need:
        raise ValueError(f"{path}: {len(raw)} bytes, need {need}")
    sig = np.frombuffer(raw[44:need], "<f8").copy()
    return int(p), int(N), int(it), sig


class ReferenceRun:
    """What one run printed: checkpoint lines, error-trial round-off, captured state."""

    def __init__(self):
        self.checkpoints: list[tuple[int, float, int | None]] = []   # (k, ms/iter, res64)
        self.trial_maxerr: list[float] = []
        self.state: tuple[int, np.ndarray] | None = None              # (k, weighted signal)
        self.returncode: int | None = None
        self.stdout_tail: list[str] = []
        self.stderr_tail: list[str] = []
        self.wall_s = 0.0

    def res64(self, k: int) -> int:
        for kk, _, r in self.checkpoints:
            if kk == k and r is not None:
                return r
        raise KeyError(f"no Res64 printed for iteration {k}")

    def ms_per_iter(self, index: int = -1) -> float:
        return self.checkpoints[index][1]


def _reader(stream, q: queue.Queue, tag: str):
    for line in iter(stream.readline, ""):
        q.put((tag, line.rstrip("\n")))
    q.put((tag, None))


def run(p: int, N: int, every: int, checkpoints: int = 1, verbose: bool = True,
        capture_state: bool = False, timeout: float = 900.0, device: int = 0) -> ReferenceRun:
    """Run ``gpuLucas -d device -f N -c every [-v] p`` until it has printed ``checkpoints``
    checkpoint lines (iterations every, 2 every, ...), then end it with SIGINT.

    capture_state: at the first checkpoint line, read the weighted signal it wrote for
    iteration ``every`` (the FFT input after ``every`` squarings)."""
    if not available():
        raise FileNotFoundError("the reference program is not built (oracle/build_ref.py)")
    if every < 2:
        raise ValueError("every must be >= 2")
    work = tempfile.mkdtemp(prefix=f"gpulucas_ref_{p}_")
    cmd = [BINARY, "-d", str(device), "-f", str(N), "-c", str(every)] + (["-v"] if verbose else []) + [str(p)]
    out = ReferenceRun()
    t0 = time.monotonic()
    proc = subprocess.Popen(cmd, cwd=work, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                            stdin=subprocess.DEVNULL, text=True, bufsize=1)
    q: queue.Queue = queue.Queue()
    threads = [threading.Thread(target=_reader, args=(proc.stdout, q, "out"), daemon=True),
               threading.Thread(target=_reader, args=(proc.stderr, q, "err"), daemon=True)]
    for t in threads:
        t.start()
    open_streams = 2
    interrupted = False
    try:
        while open_streams:
            left = timeout - (time.monotonic() - t0)
            if left <= 0:
                raise TimeoutError(f"reference run {' '.join(cmd)} exceeded {timeout:.0f} s")
            try:
                tag, line = q.get(timeout=min(left, 1.0))
            except queue.Empty:
                continue
            if line is None:
                open_streams -= 1
                continue
            tail = out.stdout_tail if tag == "out" else out.stderr_tail
            tail.append(line)
            del tail[:-40]
            if tag != "out":
                continue
            m = _ERR_LINE.search(line)
            if m and len(out.checkpoints) == 0:
                out.trial_maxerr.append(float(m.group(1)))
            m = _CP_LINE.search(line)
            if not m or interrupted:
                continue
            k = int(m.group(1))
            res = int(m.group(3), 16) if m.group(3) else None
            out.checkpoints.append((k, float(m.group(2)), res))
            if capture_state and out.state is None and k == every:
                os.kill(proc.pid, signal.SIGSTOP)
                _wait_stopped(proc.pid)
                try:
                    out.state = _grab_state(work, p, N, every)
                finally:
                    os.kill(proc.pid, signal.SIGCONT)
            if len(out.checkpoints) >= checkpoints:
                os.kill(proc.pid, signal.SIGINT)
                interrupted = True
        out.returncode = proc.wait(timeout=max(1.0, timeout - (time.monotonic() - t0)))
    except BaseException:
        if proc.poll() is None:
            os.kill(proc.pid, signal.SIGKILL)
            proc.wait()
        raise
    finally:
        out.wall_s = time.monotonic() - t0
        for t in threads:
            t.join(timeout=5)
        shutil.rmtree(work, ignore_errors=True)
    if out.returncode != 0:
        raise RuntimeError(f"reference run exited {out.returncode}:\n" + "\n".join(out.stdout_tail[-10:] +
                                                                               out.stderr_tail[-10:]))
    if len(out.checkpoints) < checkpoints:
        raise RuntimeError("reference run ended before its checkpoints:\n" + "\n".join(out.stdout_tail[-10:]))
    if capture_state and out.state is None:
        raise RuntimeError("reference run: no checkpoint state captured")
    return out


def _wait_stopped(pid: int, limit_s: float = 2.0):
    """Wait (bounded) until the kernel reports the process stopped ('T' in /proc/pid/stat)."""
    t0 = time.monotonic()
    while time.monotonic() - t0 < limit_s:
        try:
            with open(f"/proc/{pid}/stat") as f:
                if f.read().rsplit(")", 1)[1].split()[0] in ("T", "t"):
                    return
        except OSError:
            return
        time.sleep(0.002)


def _grab_state(work: str, p: int, N: int, every: int):
    """The checkpoint written at iteration every + 1 (every squarings done), from <p>.chk or,
    if a later checkpoint already rotated it, <p>.chk.bak."""
    for name in (f"{p}.chk", f"{p}.chk.bak"):
        path = os.path.join(work, name)
        if not os.path.isfile(path):
            continue
        pp, NN, it, sig = read_checkpoint(path)
        if (pp, NN, it) == (p, N, every + 1):
            return every, sig
    raise RuntimeError(f"no checkpoint for iteration {every + 1} in {work}")
