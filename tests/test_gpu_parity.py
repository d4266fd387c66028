"""GPU parity: the CUDA path through the C ABI against the oracle, bit-exact.

The loop-carried products (llint_signal) and the carry-save state (i_signal +
i_hiBitArr) after k iterations must equal the oracle's restatement of the reference
(gpuLucas.cu:845-942 mersenneIter, IrrBaseBalanced.cu:52-110 llintToIrrBal<n>) exactly:
they are integers, so any difference is a bug, not round-off.  Residues are checked
against the exact NTT oracle and the committed golden Res64 values.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))

SMALL = [(44497, 2048), (100003, 5184), (12379, 640), (1000003, 54432), (86243, 4096)]


def golden_res64():
    with open(os.path.join(HERE, "golden", "res64.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("p,N", SMALL)
@pytest.mark.parametrize("mode", [0, 1], ids=["fused", "plain"])
def test_products_and_carry_state_match_oracle(gl, orc, p, N, mode):
    with gl.Plan(p, N, mode=mode) as pl:
        o = orc.IBDWT(p, N)
        done = 0
        for step in (1, 1, 2, 6, 30):
            pl.iterate(step)
            o.iterate(step)
            done += step
            ll = pl.products()
            ref = o.ll()
            bad = np.nonzero(ll != ref)[0]
            assert bad.size == 0, f"iteration {done}: {bad.size} products differ, first {bad[:8]}"
        d, h = pl.carry_state()
        d2, h2 = o.state()
        assert (d == d2).all() and (h == h2).all()
        digits, r, z = pl.residue()
        _, r2, _, z2 = o.residue()
        assert r == r2 and z == z2
        assert r == orc.Exact(p).iterate(done).res64()


def _carry_states(orc, p, N, rng):
    """Random balanced states and the edge cases of the carry chains."""
    b, _ = orc.bits(p, N)
    b = b.astype(np.int64)
    half = (1 << (b - 1)).astype(np.int64)
    yield "random", rng.integers(-half, half).astype(np.int32), rng.integers(-128, 128, N).astype(np.int8)
    yield "zero", np.zeros(N, np.int32), np.zeros(N, np.int8)
    yield "all max (2^p - 1)", ((1 << b) - 1).astype(np.int32), np.zeros(N, np.int8)
    d = np.zeros(N, np.int32)
    d[0] = -1
    yield "minus one", d, np.zeros(N, np.int8)
    d = np.where(rng.random(N) < 0.95, half - 1, -half).astype(np.int32)
    yield "long chains", d, rng.integers(-2, 3, N).astype(np.int8)
    yield "all negative", (-half).astype(np.int32), np.full(N, -1, np.int8)
    d = np.zeros(N, np.int32)
    d[N - 1] = -1
    yield "borrow wraps", d, np.zeros(N, np.int8)


@pytest.mark.parametrize("p,N", [(44497, 2048), (4423, 256), (1000003, 54432), (2976221, 163840),
                                 (43112609, 2359296)])
@pytest.mark.parametrize("mode", [0, 1], ids=["fused", "plain"])
def test_device_residue_matches_oracle(gl, orc, p, N, mode):
    """The device normalisation (balanced rebalance, canonical digits, Res64, zero test)
    against the oracle's restatement of rebalanceIrrIntSEQGPU (IrrBaseBalanced.cu:133-169) and
    print_residue (gpuLucas.cu:1288-1352) on arbitrary carry-save states.  N = 2359296
    spans 1152 blocks of the scan, more than one pass of the one-block scan."""
    rng = np.random.default_rng(N + mode)
    with gl.Plan(p, N, mode=mode) as pl:
        for name, d, h in _carry_states(orc, p, N, rng):
            if N > 200000 and name not in ("random", "all max (2^p - 1)", "borrow wraps"):
                continue
            pl.set_carry_state(d, h, 7)
            digits, r, z = pl.residue()
            ref = orc.rebalance(p, N, d, h)
            assert (digits == ref).all(), (name, np.nonzero(digits != ref)[0][:8])
            exact_zero = name in ("zero", "all max (2^p - 1)")   # by construction
            if N <= 4096:
                assert (orc.digits_to_int(p, N, ref) == 0) == exact_zero
            assert z == exact_zero, name
            assert r == (0 if exact_zero else orc.res64_normalize(p, N, ref)), name
            assert pl.res64_zero() == (r, z)


@pytest.mark.parametrize("p,N", [(44497, 2048), (12379, 640), (86243, 4096), (100003, 5184), (300007, 15360),
                                 (600011, 32768)])
def test_resident_form_matches_oracle(gl, orc, p, N):
    """Short lengths run whole check intervals in one cluster (state and tables in
    distributed shared memory); the products equal the oracle's and the three-launch
    form's, across several launches and a state load."""
    with gl.Plan(p, N, resident=1) as pl, gl.Plan(p, N, resident=-1) as ref:
        assert pl.info.resident_ctas in (8, 16) and ref.info.resident_ctas == 0
        o = orc.IBDWT(p, N)
        for k in (1, 5, 37):
            pl.iterate(k)
            ref.iterate(k)
            o.iterate(k)
            assert (pl.products() == o.ll()).all() and (ref.products() == o.ll()).all()
        d, h = pl.carry_state()
        pl.set_carry_state(d, h, 43)   # the next iteration loads the state, then resident
        pl.iterate(20)
        o.iterate(20)
        assert (pl.products() == o.ll()).all()
        assert pl.res64() == orc.Exact(p).iterate(63).res64()


@pytest.mark.parametrize("p,N,H", [(2976221, 163840, 256), (20000000, 1179648, 2048), (43112609, 2359296, 2048),
                                   (43112609, 2359296, 1024)])
@pytest.mark.parametrize("mode", [1, 2], ids=["inplace", "inplace+prefetch"])
def test_inplace_column_passes_match(gl, orc, p, N, H, mode):
    """The in-place column DFTs (one shared-memory buffer, four CTAs per SM; power-of-two
    column lengths), with or without the bulk-copied inverse weights, give the products of
    the two-buffer form, and the oracle's."""
    with gl.Plan(p, N, col_inplace=mode, fft_h=H, autotune=0) as a, \
            gl.Plan(p, N, col_inplace=-1, fft_h=H, autotune=0) as b:
        assert b.info.smem_col == 2 * a.info.smem_col   # the forward column pass's buffer
        a.iterate(7)
        b.iterate(7)
        pa = a.products()
        assert (pa == b.products()).all()
        if N <= 163840:
            o = orc.IBDWT(p, N).iterate(7)
            assert (pa == o.ll()).all()


@pytest.mark.parametrize("p,N", [(2000003, 131072), (645131, 36864), (43112609, 2359296)],
                         ids=["depth4-W64", "depth3-W9-odd", "C3"])
@pytest.mark.parametrize("variant", [3, 4], ids=["both-two-column", "fwd-two-column+inv-prefetch"])
def test_two_column_passes_match_oracle(gl, orc, p, N, variant):
    """Two columns per CTA (col_inplace 3: each half of the block runs one column's in-place
    DFT behind its own named barrier, so one half's dicing or rounding overlaps the other
    half's DFT) gives the products of the two-buffer form and of the oracle: carry depths 4
    and 3 (ratio 15 and 17), an odd number of columns (the last CTA holds one), C3; and
    after a resume from a carry-save state, where the first forward pass loads digits and
    carries instead of dicing products.  Variant 4 pairs the two-column forward pass with the
    single-column inverse pass that prefetches its weights."""
    H = 2048
    with gl.Plan(p, N, col_inplace=variant, fft_h=H, autotune=0) as a, \
            gl.Plan(p, N, col_inplace=-1, fft_h=H, autotune=0) as b:
        assert a.info.cols_per_cta == 2 and b.info.cols_per_cta == 1
        assert a.info.fft_h == H and a.info.threads_col == 256
        o = orc.IBDWT(p, N) if N <= 163840 else None
        done = 0
        for k in (1, 6):
            a.iterate(k)
            b.iterate(k)
            done += k
            pa = a.products()
            assert (pa == b.products()).all(), f"iteration {done}"
            if o is not None:
                o.iterate(k)
                assert (pa == o.ll()).all(), f"iteration {done}"
        d, h = b.carry_state()
        b.iterate(5)
        a.set_carry_state(d, h, done)
        a.iterate(5)
        assert (a.products() == b.products()).all()
        assert a.res64() == b.res64()


@pytest.mark.parametrize("p,N", [(2000003, 131072), (645131, 36864), (43112609, 2359296)],
                         ids=["W32", "W9", "C3"])
@pytest.mark.parametrize("row_pass", [1, 2], ids=["r43-shared", "r43-l1"])
def test_row_pass_variants_match_oracle(gl, orc, p, N, row_pass):
    """The row pass compiled for radices 4, 3, 2 only (row plans 4·4·2, 3·3, 4·4·4·3·3), with
    its stage values in shared memory or read through L1, gives the products of the generic
    row pass and of the oracle."""
    H = 2048
    with gl.Plan(p, N, row_pass=row_pass, max_radix_row=4, fft_h=H, autotune=0) as a, \
            gl.Plan(p, N, row_pass=-1, max_radix_row=4, fft_h=H, autotune=0) as b:
        assert a.info.row_variant == row_pass and b.info.row_variant == -1
        if row_pass == 2:
            assert a.info.smem_row < b.info.smem_row
        a.iterate(7)
        b.iterate(7)
        pa = a.products()
        assert (pa == b.products()).all()
        if N <= 163840:
            assert (pa == orc.IBDWT(p, N).iterate(7).ll()).all()


def test_row_pass_variant_refused_for_other_radices(gl):
    """A row plan with a radix-8 stage cannot take the radix-4/3/2 row pass."""
    with pytest.raises(gl.GLError):
        gl.Plan(43112609, 2359296, row_pass=1, max_radix_row=8, fft_h=2048, autotune=0)


@pytest.mark.parametrize("p,N", [(44497, 2048), (1000003, 54432), (2976221, 163840)])
@pytest.mark.parametrize("caps", [(4, 4), (2, 2), (4, 8), (8, 2)])
def test_radix_capped_layouts_match_oracle(gl, orc, p, N, caps):
    """Line plans with smaller radices (more threads per line, for short lengths) give
    the same integer products as the oracle."""
    with gl.Plan(p, N, max_radix_col=caps[0], max_radix_row=caps[1], autotune=0, resident=-1) as pl:
        top = lambda cap: 9 if cap >= 8 else max(cap, 7)  # noqa: E731  odd radices are not capped
        assert max(pl.info.radix_h) <= top(caps[0]) and max(pl.info.radix_w) <= top(caps[1])
        o = orc.IBDWT(p, N)
        pl.iterate(9)
        o.iterate(9)
        assert (pl.products() == o.ll()).all()


@pytest.mark.parametrize("p,N", [(44497, 2048), (1000003, 54432)])
def test_dice_through_abi(gl, orc, p, N):
    """llintToBalInt<n> semantics on arbitrary products via gl_set_products."""
    rng = np.random.default_rng(p)
    ll = rng.integers(-(2**44), 2**44, N, dtype=np.int64)
    with gl.Plan(p, N) as pl:
        pl.set_products(ll, 0)
        d, h = pl.carry_state()
    d2, h2 = orc.dice(p, N, ll)
    assert (d == d2).all() and (h == h2).all()


def test_fused_equals_plain_long_run(gl):
    p, N = 1000003, 54432
    with gl.Plan(p, N, mode=0) as a, gl.Plan(p, N, mode=1) as b:
        a.iterate(700)
        b.iterate(700)
        assert (a.products() == b.products()).all()


@pytest.mark.parametrize("mode", [0, 1], ids=["fused", "plain"])
def test_golden_res64(gl, mode):
    for e in golden_res64():
        p, N, k = e["p"], e["N"], e["k"]
        if mode == 1 and k > 20000:
            continue  # the plain form runs the long ones too slowly to be worth it here
        with gl.Plan(p, N, mode=mode) as pl:
            rep = pl.iterate(k)
            _, r, z = pl.residue()
        assert f"{r:016x}" == e["res64"], (p, N, k)
        assert z == e["is_zero"]
        assert rep.max_roundoff < 0.4


def test_carry_state_resume(gl, orc):
    """Stop, export the carry-save state, resume in a fresh plan: same products."""
    p, N = 100003, 5184
    with gl.Plan(p, N) as a:
        a.iterate(300)
        d, h = a.carry_state()
        a.iterate(200)
        ref = a.products()
    with gl.Plan(p, N) as b:
        b.set_carry_state(d, h, 300)
        b.iterate(200)
        assert (b.products() == ref).all()


def test_mersenne_test_entry_points(gl):
    assert gl.mersenneTest(44497, 2048) == 1
    assert gl.mersenneTest(44501, 2048) == 0   # 44501 is prime, M44501 composite
    ms = gl.errorTest(86243, 4096)
    assert ms > 0


def test_roundoff_abort_is_reported(gl):
    """A too-small FFT length must stop with GL_ERR_ROUNDOFF, not trap or hang."""
    with gl.Plan(44497, 2048, error_limit=0.05, check_every=50) as pl:
        rep = pl.iterate(2000, check=False)
        assert rep.status == gl.GL_ERR_ROUNDOFF
        assert rep.iterations < 2000


@pytest.mark.parametrize("p,N,mode", [(44497, 2048, 0), (100003, 5184, 0), (1000003, 54432, 0), (100003, 5184, 1)])
def test_iterate_host_state_chain(gl, orc, p, N, mode):
    """gl_iterate_host from a host-held carry-save state, step after step, follows the
    oracle's iteration exactly (both forms; N = 2048 runs the resident form)."""
    o = orc.IBDWT(p, N)
    d, h = o.state()
    with gl.Plan(p, N, mode=mode) as pl:
        for k in (1, 3, 1, 10):
            d, h, rep = pl.iterate_host(d, h, k)
            o.iterate(k)
            d2, h2 = o.state()
            assert rep.status == 0 and (d == d2).all() and (h == h2).all()
        pl.set_carry_state(d, h, 15)
        assert pl.res64() == orc.Exact(p).iterate(15).res64()


@pytest.mark.parametrize("p,N,mode", [(44497, 2048, 0), (1000003, 54432, 0), (100003, 5184, 1),
                                      (43112609, 2359296, 0)])
def test_iterate_host_words_chain(gl, orc, p, N, mode):
    """gl_iterate_host_words (the state as carry-added words, digit[j] + hi[j-1]) follows the
    carry-save chain exactly: after each call the words equal the oracle's state with its
    carries added, and the products equal the oracle's (the continuation from (words, 0)
    feeds the same FFT input as (digit, hi)).  C3 is checked against the carry-save path."""
    if N > 200000:
        with gl.Plan(p, N) as a, gl.Plan(p, N) as b:
            d = np.zeros(N, np.int32)
            d[0] = 4                      # S0 = 4
            h = np.zeros(N, np.int8)
            w = d.copy()
            for k in (1, 4):
                w, rep = a.iterate_host_words(w, k)
                d, h, _ = b.iterate_host(d, h, k)
                assert rep.status == 0 and (w == d + np.roll(h.astype(np.int32), 1)).all()
            assert (a.products() == b.products()).all()
        return
    o = orc.IBDWT(p, N)
    d, h = o.state()
    w = d + np.roll(h.astype(np.int32), 1)
    with gl.Plan(p, N, mode=mode) as pl:
        for k in (1, 3, 10):
            w, rep = pl.iterate_host_words(w, k)
            o.iterate(k)
            d2, h2 = o.state()
            assert rep.status == 0 and (w == d2 + np.roll(h2.astype(np.int32), 1)).all()
            assert (pl.products() == o.ll()).all()
        assert pl.res64() == orc.Exact(p).iterate(14).res64()


@pytest.mark.parametrize("p,N,mode", [(1000003, 54432, 0), (100003, 5184, 1), (44497, 2048, 0)])
def test_iterate_host_pinned_buffers(gl, orc, p, N, mode):
    """Pinned host buffers, updated in place step after step: the same states as the
    oracle."""
    import ctypes

    import torch
    o = orc.IBDWT(p, N)
    d0, h0 = o.state()
    d = torch.from_numpy(np.ascontiguousarray(d0, np.int32)).pin_memory()
    h = torch.from_numpy(np.ascontiguousarray(h0, np.int8)).pin_memory()
    dp, hp = ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(h.data_ptr())
    rep = gl.IterReport()
    with gl.Plan(p, N, mode=mode) as pl:
        for k in (1, 4, 1):
            assert gl.lib.gl_iterate_host(pl._h, dp, hp, k, dp, hp, ctypes.byref(rep)) == 0
            o.iterate(k)
            d2, h2 = o.state()
            assert (d.numpy() == d2).all() and (h.numpy() == h2).all()


@pytest.mark.parametrize("p,N", [(1000003, 54432), (43112609, 2359296)])
def test_iterate_host_words_pinned_graph(gl, orc, p, N):
    """Pinned buffers and one iteration per call take the captured-step path (one graph per
    plan and buffer pair): in place step after step, then into a second buffer (the graph
    is rebuilt), the words equal those of the same steps through pageable buffers, and
    the iteration count and products follow."""
    import ctypes

    import torch
    w0 = np.zeros(N, np.int32)
    w0[0] = 4
    a = torch.from_numpy(w0.copy()).pin_memory()
    b = torch.empty(N, dtype=torch.int32).pin_memory()
    ap, bp = ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr())
    rep = gl.IterReport()
    with gl.Plan(p, N) as pl, gl.Plan(p, N) as ref:
        w = w0.copy()
        for step in range(3):
            assert gl.lib.gl_iterate_host_words(pl._h, ap, 1, ap, ctypes.byref(rep)) == 0
            assert rep.iterations == 1 and rep.total_iterations == step + 1
            w, _ = ref.iterate_host_words(w, 1)
            assert (a.numpy() == w).all(), step
        assert gl.lib.gl_iterate_host_words(pl._h, ap, 1, bp, ctypes.byref(rep)) == 0
        w, _ = ref.iterate_host_words(w, 1)
        assert (b.numpy() == w).all()
        assert (pl.products() == ref.products()).all()
        if N <= 163840:
            o = orc.IBDWT(p, N).iterate(4)
            d, h = o.state()
            assert (b.numpy() == d + np.roll(h.astype(np.int32), 1)).all()


def test_host_steps_switch_between_words_and_pair(gl, orc):
    """One plan alternating the two pinned host-state steps (carry-save pair, words, pair,
    words): each call rebuilds the plan's captured step for its kind and buffers, and
    every state equals the oracle's."""
    import ctypes

    import torch
    p, N = 1000003, 54432
    o = orc.IBDWT(p, N)
    d0, h0 = o.state()
    d = torch.from_numpy(np.ascontiguousarray(d0, np.int32)).pin_memory()
    h = torch.from_numpy(np.ascontiguousarray(h0, np.int8)).pin_memory()
    w = torch.empty(N, dtype=torch.int32).pin_memory()
    dp, hp, wp = (ctypes.c_void_p(t.data_ptr()) for t in (d, h, w))
    rep = gl.IterReport()
    with gl.Plan(p, N) as pl:
        for step in range(4):
            if step % 2 == 0:
                assert gl.lib.gl_iterate_host(pl._h, dp, hp, 1, dp, hp, ctypes.byref(rep)) == 0
                o.iterate(1)
                d2, h2 = o.state()
                assert (d.numpy() == d2).all() and (h.numpy() == h2).all(), step
                w.copy_(torch.from_numpy(d2 + np.roll(h2.astype(np.int32), 1)))
            else:
                assert gl.lib.gl_iterate_host_words(pl._h, wp, 1, wp, ctypes.byref(rep)) == 0
                o.iterate(1)
                d2, h2 = o.state()
                assert (w.numpy() == d2 + np.roll(h2.astype(np.int32), 1)).all(), step
                d.copy_(torch.from_numpy(d2))
                h.copy_(torch.from_numpy(h2))
            assert rep.status == 0 and rep.total_iterations == step + 1
        assert (pl.products() == o.ll()).all()


def test_bounded_wait_times_out_and_device_stays_usable(gl, orc):
    """A kernel waiting on a barrier that nothing completes gives up after its bound,
    the host reads GL_ERR_TIMEOUT, and the context keeps working (no trap, no hang)."""
    assert gl.lib.gl_selftest_bounded_wait(0, 1000) == gl.GL_ERR_TIMEOUT
    with gl.Plan(44497, 2048) as pl:
        pl.iterate(100)
        assert pl.res64() == orc.Exact(44497).iterate(100).res64()


def test_plans_with_different_layouts_coexist(gl):
    """Two live plans of different layouts (autotuned and forced) interleave correctly."""
    p, N = 2976221, 163840
    with gl.Plan(p, N) as a, gl.Plan(p, N, fft_h=640, autotune=0) as b:
        for _ in range(3):
            a.iterate(50)
            b.iterate(50)
        assert (a.products() == b.products()).all()


def test_find_signal_size(gl, orc):
    """findSignalSize: a usable N for p, round-off of the trial below 0.30."""
    p = 1000003
    N, ms, err = gl.find_signal_size(p)
    assert N % 2 == 0 and p // N <= 21 and err < 0.30 and ms > 0
    with gl.Plan(p, 0) as pl:
        assert pl.info.N == N
        pl.iterate(300)
        assert pl.res64() == orc.Exact(p).iterate(300).res64()


def test_fp64_probes(gl):
    """The DFMA peak probe (the roofline denominator) and the butterfly issue-rate probe
    run and report plausible rates: the butterfly code issues FP64 instructions no faster
    than independent DFMA chains do."""
    peak = gl.probe_fp64_peak(0, 50.0)
    bfly = gl.probe_fp64_butterfly(0, 50.0)
    assert 0.3 < peak < 5.0                       # TFLOP/s
    assert 0.2 * peak * 0.5e12 < bfly < 1.05 * peak * 0.5e12
