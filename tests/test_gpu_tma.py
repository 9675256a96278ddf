"""Bulk tensor (TMA) tile paths of the shared-memory point kernels against
the per-cell tile loops they replace for tiles that do not wrap.

The interpolation stages the same grid cells either way, so its results are
bit-identical; the spread adds the same tile values to the grid in a
different order (one bulk reduce-add instead of one atomic per cell), so it
agrees to FP32 round-off (5e-6 relative l2 after deconvolution).  No bounded wait may have given up."""
import ctypes
import os

import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def jf(native):
    import jax_finufft_gb300

    return jax_finufft_gb300


def _run(fn, tma):
    old = os.environ.get("GBN_DISABLE_TMA")
    os.environ["GBN_DISABLE_TMA"] = "0" if tma else "1"
    try:
        out = fn()
        torch.cuda.synchronize()
        return out
    finally:
        if old is None:
            del os.environ["GBN_DISABLE_TMA"]
        else:
            os.environ["GBN_DISABLE_TMA"] = old


CASES = [((256, 200), 50000, 1e-6, None, 1),
         ((64, 48, 40), 40000, 1e-5, None, 1),
         ((64, 64, 64), 60000, 1e-6, (8, 8, 8), 1),
         ((96, 80), 30000, 1e-5, (64, 64), 3),
         ((40, 40, 40), 20000, 1e-3, None, 2)]


@pytest.mark.parametrize("shape, M, eps, bins, T", CASES)
def test_tma_matches_cell_loops(jf, shape, M, eps, bins, T):
    from jax_finufft_gb300.options import Opts

    rng = np.random.default_rng(31 + M % 97)
    dim = len(shape)
    # half uniform, half clustered near the origin (many interior tiles and
    # several subproblems per bin)
    pts = []
    for _ in range(dim):
        a = np.concatenate([rng.uniform(-np.pi, np.pi, M // 2), rng.normal(0, 0.3, M - M // 2)])
        pts.append(torch.tensor(a.astype(np.float32), device=DEV))
    kw = {}
    if bins is not None:
        kw = dict(zip(["gpu_binsizex", "gpu_binsizey", "gpu_binsizez"], bins))
    opts = Opts(gpu_method=2, **kw)
    c = torch.tensor((rng.standard_normal((T, M)) + 1j * rng.standard_normal((T, M)))
                     .astype(np.complex64), device=DEV)
    f = torch.tensor((rng.standard_normal((T,) + shape) + 1j * rng.standard_normal((T,) + shape))
                     .astype(np.complex64), device=DEV)
    src1 = c if T > 1 else c[0]
    src2 = f if T > 1 else f[0]
    for fn in (lambda: jf.nufft1(shape, src1, *pts, eps=eps, opts=opts),):
        a, b = _run(fn, True), _run(fn, False)
        # FP32 addition order in global memory; deconvolution amplifies it
        # at the edge modes (still well below eps)
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 5e-6
    fn2 = lambda: jf.nufft2(src2, *pts, eps=eps, opts=opts)
    a, b = _run(fn2, True), _run(fn2, False)
    assert torch.equal(a, b)


def test_no_wait_gave_up(native):
    n = ctypes.c_longlong(-1)
    assert native.gbn_wait_timeouts(ctypes.byref(n), 0) == 0
    assert n.value == 0


def test_gave_up_wait_is_an_error(jf, native):
    """A bounded wait that gave up makes the next call on the device return
    GBN_ERR_CUDA (lib/kernels.cc.cu:70-79 turns a failed execute into an
    error); the flag is raised from the host, no wait is made to run out."""
    from jax_finufft_gb300 import _native

    rng = np.random.default_rng(5)
    x = [torch.tensor(rng.uniform(-np.pi, np.pi, 2000).astype(np.float32), device=DEV)
         for _ in range(2)]
    f = torch.tensor((rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32)))
                     .astype(np.complex64), device=DEV)
    good = jf.nufft2(f, *x, eps=1e-5)
    torch.cuda.synchronize()
    native.gbn_debug_raise_wait_timeout()
    with pytest.raises(_native.NufftError) as err:
        jf.nufft2(f, *x, eps=1e-5)
    assert err.value.code == 3 and "wait gave up" in str(err.value)
    # reported once: the next call runs and agrees with the first
    again = jf.nufft2(f, *x, eps=1e-5)
    torch.cuda.synchronize()
    assert torch.equal(good, again)
    # the plan API reports it the same way
    opts = _native.default_opts()
    nm = (ctypes.c_int64 * 3)(32, 32, 1)
    plan = ctypes.c_void_p()
    _native.check(native.gbnf_makeplan(2, 2, nm, -1, 1, 1e-5, ctypes.byref(plan),
                                       ctypes.byref(opts), None))
    try:
        _native.check(native.gbnf_setpts(plan, 2000, ctypes.c_void_p(x[1].data_ptr()),
                                         ctypes.c_void_p(x[0].data_ptr()), None, 0, None, None,
                                         None))
        c = torch.empty(2000, dtype=torch.complex64, device=DEV)
        native.gbn_debug_raise_wait_timeout()
        assert native.gbn_execute(plan, ctypes.c_void_p(c.data_ptr()),
                                  ctypes.c_void_p(f.data_ptr())) == 3
        assert native.gbn_execute(plan, ctypes.c_void_p(c.data_ptr()),
                                  ctypes.c_void_p(f.data_ptr())) == 0
        torch.cuda.synchronize()
        assert torch.equal(c, good)
    finally:
        native.gbn_destroy(plan)
