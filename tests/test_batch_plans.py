"""Line plans of batch members.  A batch runs one column or one row pair per CTA, and its
members' lines are short (tens to hundreds of points), so a stage's butterflies often
leave the last warp partly empty; a warp issues each FP64 instruction for all 32 lanes.
A member's plans are therefore chosen by the FP64 instructions issued, not by the work
alone.  Checked without a GPU through gl_plan_describe."""
import math

import pytest


def stage_ops(r, first):
    """FP64 instructions per point of a stage of radix r (the first stage has constant
    twiddles only; later radix 8, 4, 3 stages are in ratio form, 2 and 16 layered, 5 and
    7 a complex product per input and DFT_R)."""
    pow2 = r & (r - 1) == 0
    if not first and r in (8, 4, 3):
        return {8: 66.0, 4: 22.0, 3: 16.0}[r] / r
    if pow2:
        return 3.0 * int(math.log2(r)) if not first else {2: 2.0, 4: 4.0, 8: 6.5, 16: 9.25}[r]
    return {3: 14.0, 5: 36.0, 7: 72.0}[r] / r + (0.0 if first else 4.0 * (r - 1) / r)


def issued(L, radices, nlines):
    total = 0.0
    for s, r in enumerate(radices):
        nb = nlines * L // r
        total += stage_ops(r, s == 0) * (-(-nb // 32) * 32) / nb
    return total


def canonical(L):
    out, m = [], L
    for q in (8, 4, 2, 3, 5, 7):
        while m % q == 0:
            out.append(q)
            m //= q
    assert m == 1
    return out


def members():
    from gpulucas_gb300 import workloads
    ps = workloads.batch_exponents()
    return ps[::8]  # 32 of the 256 exponents, spread over the range


@pytest.mark.parametrize("p", members())
def test_batch_member_plans_issue_no_more_than_canonical(gl, p):
    N = gl.smallest_signal_size(p, 19.5)
    info = gl.describe(p, N, batch_layout=1)
    H, W = info.fft_h, info.fft_w
    rw = [r for r in info.radix_w if r]
    rh = [r for r in info.radix_h if r]
    assert H * W == N // 2
    assert math.prod(rw) == W and math.prod(rh) == H
    assert set(rw + rh) <= {2, 3, 4, 5, 7, 8} and len(rw) <= 8 and len(rh) <= 8
    # rows: a CTA takes the row pair (two lines); columns: one line
    assert issued(W, rw, 2) <= issued(W, canonical(W), 2) + 1e-9
    assert issued(H, rh, 1) <= issued(H, canonical(H), 1) + 1e-9


def test_batch_member_plan_fills_warps_on_a_320_point_column(gl):
    """A 320-point column as 8·8·5 has 40, 40 and 64 butterflies per stage (warps 62.5 %,
    62.5 %, 100 % full); the plan chosen issues fewer FP64 instructions than that."""
    from gpulucas_gb300 import workloads
    for p in workloads.batch_exponents():
        N = gl.smallest_signal_size(p, 19.5)
        info = gl.describe(p, N, batch_layout=1)
        if info.fft_h == 320:
            rh = [r for r in info.radix_h if r]
            assert issued(320, rh, 1) < issued(320, [8, 8, 5], 1)
            return
    pytest.skip("no member with 320-point columns")
