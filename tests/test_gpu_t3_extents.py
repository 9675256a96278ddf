"""Type-3 setpts with declared extents (gbn_set_t3_extents).

The reference's type-3 setpts (cuFINUFFT's, behind lib/cufinufft_wrapper.cc:
63-73) measures the point extents on the host to size its grid; with
declared extents this library's setpts skips that host round trip.  Checked
here through the C ABI:
  * extents equal to the measured ones give the measured path's outputs
    (to FP32 rounding: tiles of one bin reach the grid by float reduce-adds
    in a run-dependent order);
  * wider extents give a larger grid and stay within the FP32 tolerance of
    the FP64 direct sum (oracle/direct.py, rtol 1e-3 for complex64 type 3 as
    tests/ops_test.py:120 uses, in relative l2);
  * a source outside its declared extent makes the next API call return
    GBN_ERR_ARGS, and the call after it succeeds again;
  * setpts + execute are captured into a CUDA graph and replayed with the
    eager result (to FP32 rounding).
"""
import ctypes

import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu

D3 = ctypes.c_double * 3


def _plan(lib, native, dim, stream):
    opts = native.default_opts()
    p = ctypes.c_void_p()
    nm = (ctypes.c_int64 * 3)(1, 1, 1)
    native.check(lib.gbnf_makeplan(3, dim, nm, -1, 1, ctypes.c_float(1e-4), ctypes.byref(p),
                                   ctypes.byref(opts), ctypes.c_void_p(stream)))
    return p


def _data(seed, dim, M, N):
    rng = np.random.default_rng(seed)
    x = [rng.uniform(-3.0, 3.0, M).astype(np.float32) for _ in range(dim)]
    s = [rng.uniform(-20.0, 20.0, N).astype(np.float32) for _ in range(dim)]
    c = (rng.normal(size=M) + 1j * rng.normal(size=M)).astype(np.complex64)
    return x, s, c


def _ptrs(ts, dim):
    return [ctypes.c_void_p(t.data_ptr()) for t in ts] + [None] * (3 - dim)


def _run(lib, native, p, xd, sd, cd, out, dim):
    M, N = xd[0].numel(), sd[0].numel()
    rc = lib.gbnf_setpts(p, M, *_ptrs(xd, dim), N, *_ptrs(sd, dim))
    if rc >= 2:
        return rc
    return lib.gbn_execute(p, ctypes.c_void_p(cd.data_ptr()), ctypes.c_void_p(out.data_ptr()))


def _ext(x, s, dim, pad=0.0):
    xl = D3(*[float(v.min()) - pad for v in x] + [0.0] * (3 - dim))
    xh = D3(*[float(v.max()) + pad for v in x] + [0.0] * (3 - dim))
    sl = D3(*[float(v.min()) - pad for v in s] + [0.0] * (3 - dim))
    sh = D3(*[float(v.max()) + pad for v in s] + [0.0] * (3 - dim))
    return xl, xh, sl, sh


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_declared_extents_match_measured(dim):
    from jax_finufft_gb300 import _native
    from oracle import direct

    lib = _native.load()
    st = torch.cuda.current_stream().cuda_stream
    M, N = 3000, 2500
    x, s, c = _data(5 + dim, dim, M, N)
    xd = [torch.tensor(v, device="cuda") for v in x]
    sd = [torch.tensor(v, device="cuda") for v in s]
    cd = torch.tensor(c, device="cuda")
    ref_out = torch.empty(N, dtype=torch.complex64, device="cuda")
    p = _plan(lib, _native, dim, st)
    try:
        _native.check(_run(lib, _native, p, xd, sd, cd, ref_out, dim))
        out = torch.empty_like(ref_out)
        _native.check(lib.gbn_set_t3_extents(p, *_ext(x, s, dim)))
        _native.check(_run(lib, _native, p, xd, sd, cd, out, dim))
        torch.cuda.synchronize()
        d = rel_l2(out.cpu().numpy(), ref_out.cpu().numpy())
        assert d < 1e-6, d
        # wider extents: a larger grid, the same accuracy
        _native.check(lib.gbn_set_t3_extents(p, *_ext(x, s, dim, pad=1.5)))
        _native.check(_run(lib, _native, p, xd, sd, cd, out, dim))
        torch.cuda.synchronize()
        exact = direct.type3(c.astype(np.complex128), [v.astype(np.float64) for v in x],
                             [v.astype(np.float64) for v in s], iflag=-1)
        assert rel_l2(out.cpu().numpy(), exact) < 1e-3
        # back to measured extents
        _native.check(lib.gbn_set_t3_extents(p, None, None, None, None))
        _native.check(_run(lib, _native, p, xd, sd, cd, out, dim))
        torch.cuda.synchronize()
        d = rel_l2(out.cpu().numpy(), ref_out.cpu().numpy())
        assert d < 1e-6, d
    finally:
        lib.gbn_destroy(p)


def test_point_outside_declared_extents_is_an_error():
    from jax_finufft_gb300 import _native

    lib = _native.load()
    st = torch.cuda.current_stream().cuda_stream
    dim, M, N = 2, 2000, 1000
    x, s, c = _data(41, dim, M, N)
    xd = [torch.tensor(v, device="cuda") for v in x]
    sd = [torch.tensor(v, device="cuda") for v in s]
    cd = torch.tensor(c, device="cuda")
    out = torch.empty(N, dtype=torch.complex64, device="cuda")
    p = _plan(lib, _native, dim, st)
    try:
        xl, xh, sl, sh = _ext(x, s, dim)
        xh[0] = float(x[0].max()) - 0.5  # some sources lie beyond the declared upper bound
        _native.check(lib.gbn_set_t3_extents(p, xl, xh, sl, sh))
        lib.gbnf_setpts(p, M, *_ptrs(xd, dim), N, *_ptrs(sd, dim))
        torch.cuda.synchronize()  # the check kernel has run
        rc = lib.gbn_execute(p, ctypes.c_void_p(cd.data_ptr()), ctypes.c_void_p(out.data_ptr()))
        assert rc == 2
        assert "outside the extents" in _native.last_error()
        # the flag was taken: calls with valid extents succeed again
        _native.check(lib.gbn_set_t3_extents(p, *_ext(x, s, dim)))
        _native.check(_run(lib, _native, p, xd, sd, cd, out, dim))
        torch.cuda.synchronize()
        # invalid declarations are refused on the host
        bad = D3(1.0, 0.0, 0.0)
        assert lib.gbn_set_t3_extents(p, bad, D3(0.0, 0.0, 0.0), sl, sh) == 2
    finally:
        lib.gbn_destroy(p)


def test_setpts_and_execute_capture_into_a_graph():
    from jax_finufft_gb300 import _native

    lib = _native.load()
    stream = torch.cuda.Stream()
    dim, M, N = 3, 4000, 3000
    x, s, c = _data(77, dim, M, N)
    with torch.cuda.stream(stream):
        xd = [torch.tensor(v, device="cuda") for v in x]
        sd = [torch.tensor(v, device="cuda") for v in s]
        cd = torch.tensor(c, device="cuda")
        eager = torch.empty(N, dtype=torch.complex64, device="cuda")
        graphed = torch.zeros_like(eager)
    stream.synchronize()
    p = _plan(lib, _native, dim, stream.cuda_stream)
    try:
        _native.check(lib.gbn_set_t3_extents(p, *_ext(x, s, dim, pad=0.25)))
        # first call outside the capture: makes the inner plan and buffers
        _native.check(_run(lib, _native, p, xd, sd, cd, eager, dim))
        stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            _native.check(_run(lib, _native, p, xd, sd, cd, graphed, dim))
        g.replay()
        torch.cuda.synchronize()
        d = rel_l2(graphed.cpu().numpy(), eager.cpu().numpy())
        assert d < 1e-6, d
    finally:
        lib.gbn_destroy(p)
