"""The C-ABI library without a GPU: it loads, exports what include/gpulucas.h declares,
validates arguments with status codes (never exit(), unlike cuda_safecalls.h:37-98),
and picks sane FFT layouts (gl_plan_describe)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpulucas.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+([A-Za-z_][A-Za-z0-9_]*)\s*\(", src, re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(gl):
    names = header_functions()
    assert len(names) >= 20
    lib = ctypes.CDLL(gl.LIB_PATH)
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(gl.ABI_SYMBOLS) == names
    out = subprocess.run(["nm", "-D", "--defined-only", gl.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(names) <= exported


def test_library_is_built_for_sm_103a(gl):
    from gpulucas_gb300 import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)


def test_status_strings(gl):
    for code in range(0, -12, -1):
        assert gl.error_string(code)


@pytest.mark.parametrize("p,N,code", [(44497, 2047, -1), (44497, 2, -1), (1000, 2048, -1),
                                      (50000, 2048, -2), (60013, 2 * 11 * 256, -3)])
def test_describe_rejects(gl, p, N, code):
    with pytest.raises(gl.GLError) as ei:
        gl.describe(p, N)
    assert ei.value.status == code


@pytest.mark.parametrize("p,N", [(44497, 2048), (2976221, 163840), (43112609, 2359296), (100003, 5184),
                                 (1000003, 54432), (2999999, 154350), (12379, 640), (300007, 15360)])
@pytest.mark.parametrize("mode", [0, 1])
def test_describe_layouts(gl, p, N, mode):
    info = gl.describe(p, N, mode=mode)
    M = N // 2
    assert info.lo_bits == p // N and info.hi_bits == p // N + 1
    assert info.carry_depth == gl.setSliceAndDice(p, N)
    if mode == 0:
        assert info.fft_w * info.fft_h == M
        assert info.fft_w % info.cols_per_cta == 0
        rw = [r for r in info.radix_w if r]
        rh = [r for r in info.radix_h if r]
        prod = lambda xs: eval("*".join(map(str, xs))) if xs else 1  # noqa: E731
        assert prod(rw) == info.fft_w and prod(rh) == info.fft_h
        assert set(rw + rh) <= {2, 3, 4, 5, 7, 8}
        assert info.cols_per_cta == 1
        ls = lambda L: L + L // 16 + 1  # noqa: E731  padded line stride
        assert info.smem_col == 2 * ls(info.fft_h) * 16 <= 110 * 1024
        # four line buffers plus the row pass's stage values, copied in by one bulk copy
        # slots per butterfly position: radix 8, 4, 3 in ratio form (8, 4, 4), radix 2 one
        # complex value, 5 and 7 one per twiddled input
        values = lambda r: {2: 1, 3: 4, 4: 4, 8: 8, 16: 8}.get(r, r - 1)  # noqa: E731
        table, ns = 1, 1
        for i, r in enumerate(rw):
            if i:
                table += values(r) * ns
            ns *= r
        assert info.smem_row == 4 * ls(info.fft_w) * 16 + 16 * table <= 112 * 1024
        assert 64 <= info.threads_col <= 256 and info.threads_col % 32 == 0
        assert 64 <= info.threads_row <= 256 and info.threads_row % 32 == 0


def test_row_block_balances_stages(gl):
    """A row CTA (two lines of W points) gets the smallest block that minimises the stages'
    rounds weighted by radix: W = 576 (8, 8, 3, 3) runs 192 threads, so its radix-3 stages
    (384 butterflies) take two even rounds."""
    info = gl.describe(43112609, 2359296)
    rw = [r for r in info.radix_w if r]
    assert info.fft_w == 576 and rw == [8, 8, 3, 3] and info.threads_row == 192
    for p, N in [(2976221, 163840), (1000003, 54432), (300007, 15360)]:
        info = gl.describe(p, N)
        t = info.threads_row
        rw = [r for r in info.radix_w if r]
        cost = lambda t: sum(-(-2 * info.fft_w // r // t) * r for r in rw)  # noqa: E731
        assert all(cost(t) <= cost(u) for u in range(64, 257, 32) if u >= t)


def test_plan_without_gpu_reports_status(gl):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gl.GLError) as ei:
        gl.Plan(44497, 2048)
    assert ei.value.status == gl.GL_ERR_NODEVICE


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the header's structs have the C compiler's sizes and offsets."""
    import ctypes
    import shutil
    import subprocess

    import gpulucas_gb300 as gl
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    pairs = {"gl_plan_opts": gl.PlanOpts, "gl_plan_info": gl.PlanInfo, "gl_iter_report": gl.IterReport,
             "gl_result": gl.Result, "gl_batch_info": gl.BatchInfo, "gl_server_opts": gl.ServerOpts,
             "gl_completion": gl.Completion, "gl_server_stats": gl.ServerStats, "gl_server_engine": gl.ServerEngine}
    inc = os.path.join(ROOT, "include")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gpulucas.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    for cname, py in pairs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)
