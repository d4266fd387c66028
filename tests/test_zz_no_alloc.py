"""gl_iterate_noalloc: LL iterations for callers that may not allocate device memory.

Some callers cannot call cudaMalloc (their framework's memory pool owns the device,
or an allocation would stall work they share the GPU with).  They hand the library
device buffers for the products and gl_iterate_noalloc runs the iterations with its
own work arrays in a static device array.  These tests call it through the C ABI on
caller-owned buffers and compare its products with those of the plan-based
entry point (gl_set_products + gl_iterate + gl_get_products): integers, so they must
be equal, on two calls in a row.  The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan_products(gl, p, N, ll0, k, mode):
    with gl.Plan(p, N, mode=mode) as pl:
        pl.set_products(ll0, 0)
        pl.iterate(k)
        return pl.products()


@pytest.mark.parametrize("p,N,k", [(44497, 2048, 25), (100003, 5184, 12), (1000003, 54432, 6)])
def test_noalloc_matches_plan_on_two_calls(gl, p, N, k):
    import torch
    torch.cuda.init()
    stream = torch.cuda.current_stream().cuda_stream
    ll0 = np.zeros(N, np.int64)
    ll0[0] = 4
    d_in = torch.from_numpy(ll0).cuda()
    d_mid = torch.empty_like(d_in)
    d_out = torch.empty_like(d_in)
    torch.cuda.synchronize()
    e1 = gl.iterate_noalloc(p, N, d_in.data_ptr(), d_mid.data_ptr(), k, stream)
    e2 = gl.iterate_noalloc(p, N, d_mid.data_ptr(), d_out.data_ptr(), k, stream)
    torch.cuda.synchronize()
    mid = d_mid.cpu().numpy()
    out = d_out.cpu().numpy()
    for mode in (gl.MODE_PLAIN, gl.MODE_FUSED):
        assert np.array_equal(mid, _plan_products(gl, p, N, ll0, k, mode))
        assert np.array_equal(out, _plan_products(gl, p, N, ll0, 2 * k, mode))
    assert 0.0 <= e1 < 0.4 and 0.0 <= e2 < 0.4


def test_noalloc_in_place_and_switching_tests(gl):
    """Same buffer in and out, and a different (p, N) between calls (tables reloaded)."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    for p, N in [(12379, 640), (44497, 2048), (12379, 640)]:
        ll0 = np.zeros(N, np.int64)
        ll0[0] = 4
        d = torch.from_numpy(ll0).cuda()
        gl.iterate_noalloc(p, N, d.data_ptr(), d.data_ptr(), 40, stream)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), _plan_products(gl, p, N, ll0, 40, gl.MODE_PLAIN))


def test_noalloc_rejects_sizes_above_limit(gl):
    import torch
    N = 2 * gl.NOALLOC_MAX_N
    d = torch.zeros(N, dtype=torch.int64, device="cuda")
    err = ctypes.c_double()
    rc = gl.lib.gl_iterate_noalloc(19 * N + 1, N, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()), 1,
                                   ctypes.byref(err), None)
    assert rc == gl.GL_ERR_TOO_LARGE
    assert "65536" in gl.error_string(rc)


def test_noalloc_rejects_partly_overlapping_buffers(gl):
    """ll_in and ll_out may be the same buffer, but not overlap in part (the copy between
    them would be undefined)."""
    import torch
    N = 2048
    d = torch.zeros(2 * N, dtype=torch.int64, device="cuda")
    err = ctypes.c_double()
    base = d.data_ptr()
    for shift in (1, N - 1):
        rc = gl.lib.gl_iterate_noalloc(44497, N, ctypes.c_void_p(base), ctypes.c_void_p(base + 8 * shift), 1,
                                       ctypes.byref(err), None)
        assert rc == gl.GL_ERR_ARG, shift


def test_noalloc_refuses_a_capturing_stream(gl):
    """The call waits for its stream, so on a stream that is being captured into a CUDA
    graph it returns GL_ERR_ARG and enqueues nothing; the next call on a plain stream
    works as before."""
    import torch
    p, N = 44497, 2048
    ll0 = np.zeros(N, np.int64)
    ll0[0] = 4
    d = torch.from_numpy(ll0).cuda()
    err = ctypes.c_double()
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    rcs = []
    with torch.cuda.graph(graph, stream=side):
        rcs.append(gl.lib.gl_iterate_noalloc(p, N, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()), 3,
                                             ctypes.byref(err), ctypes.c_void_p(side.cuda_stream)))
        d.add_(0)
    assert rcs == [gl.GL_ERR_ARG]
    del graph
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), ll0)
    gl.iterate_noalloc(p, N, d.data_ptr(), d.data_ptr(), 3, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), _plan_products(gl, p, N, ll0, 3, gl.MODE_PLAIN))
