"""Edge cases through the public API: empty point sets and mode sets, a
single point or mode, points far outside one period and at the period's
ends, non-finite coordinates (folded to 0, as the CPU restatement does),
and the bounded device waits still at zero afterwards."""
import ctypes

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


@pytest.fixture(scope="module")
def cn(oracle_lib):
    from oracle import cpu_nufft

    return cpu_nufft


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_empty_point_sets(jf, ndim):
    shape = (8, 6, 4)[:ndim]
    x = [torch.zeros(0, device=DEV) for _ in range(ndim)]
    c = torch.zeros(0, dtype=torch.complex64, device=DEV)
    f1 = jf.nufft1(shape, c, *[v.float() for v in x], eps=1e-5)
    assert f1.shape == shape and torch.count_nonzero(f1) == 0
    f = torch.ones(shape, dtype=torch.complex64, device=DEV)
    c2 = jf.nufft2(f, *[v.float() for v in x], eps=1e-5)
    assert c2.shape == (0,)
    s = [torch.zeros(5, device=DEV) for _ in range(ndim)]
    f3 = jf.nufft3(c, *[v.float() for v in x], *[v.float() for v in s], eps=1e-5)
    assert f3.shape == (5,) and torch.count_nonzero(f3) == 0


def test_empty_targets_type3(jf):
    x = [torch.rand(50, device=DEV) for _ in range(2)]
    c = torch.ones(50, dtype=torch.complex64, device=DEV)
    s = [torch.zeros(0, device=DEV) for _ in range(2)]
    assert jf.nufft3(c, *x, *s, eps=1e-5).shape == (0,)


@pytest.mark.parametrize("single", [True, False])
def test_single_point_and_single_mode(jf, cn, single):
    rdt, cdt = (np.float32, np.complex64) if single else (np.float64, np.complex128)
    eps = 1e-5 if single else 1e-10
    tol = 5 * max(eps, 1e-6) if single else 5 * eps
    rng = np.random.default_rng(3)
    x = [rng.uniform(-np.pi, np.pi, 1).astype(rdt) for _ in range(2)]
    c = np.array([1.0 - 2.0j], dtype=cdt)
    out = jf.nufft1((17, 12), T(c), *[T(v) for v in x], eps=eps).cpu().numpy()
    ref = cn.nufft1((17, 12), c, *x, eps=eps)
    assert rel_l2(out, ref) < tol
    f = np.array([[2.0 + 1.0j]], dtype=cdt)
    xs = [rng.uniform(-np.pi, np.pi, 300).astype(rdt) for _ in range(2)]
    out2 = jf.nufft2(T(f), *[T(v) for v in xs], eps=eps).cpu().numpy()
    ref2 = cn.nufft2(f, *xs, eps=eps)
    assert rel_l2(out2, ref2) < tol


@pytest.mark.parametrize("ty", [1, 2])
def test_far_and_boundary_coordinates(jf, cn, ty):
    rng = np.random.default_rng(4)
    M = 2000
    pts = [np.concatenate([rng.uniform(-np.pi, np.pi, M - 8),
                           np.array([np.pi, -np.pi, np.nextafter(np.pi, 0), 1e4, -1e4,
                                     123456.789, -3 * np.pi, 7 * np.pi])])
           for _ in range(3)]
    shape = (20, 18, 16)
    if ty == 1:
        c = rng.normal(size=M) + 1j * rng.normal(size=M)
        out = jf.nufft1(shape, T(c), *[T(v) for v in pts], eps=1e-9).cpu().numpy()
        ref = cn.nufft1(shape, c, *pts, eps=1e-9)
    else:
        f = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        out = jf.nufft2(T(f), *[T(v) for v in pts], eps=1e-9).cpu().numpy()
        ref = cn.nufft2(f, *pts, eps=1e-9)
    assert rel_l2(out, ref) < 5e-9


def test_non_finite_coordinates_fold_to_zero(jf, cn):
    rng = np.random.default_rng(5)
    M = 500
    x = rng.uniform(-np.pi, np.pi, M)
    y = rng.uniform(-np.pi, np.pi, M)
    x[:3] = [np.nan, np.inf, -np.inf]
    c = rng.normal(size=M) + 1j * rng.normal(size=M)
    out = jf.nufft1((16, 14), T(c), T(x), T(y), eps=1e-9).cpu().numpy()
    ref = cn.nufft1((16, 14), c, x, y, eps=1e-9)
    assert np.isfinite(out).all()
    assert rel_l2(out, ref) < 5e-9
    x0 = x.copy()
    x0[:3] = 0.0
    ref0 = cn.nufft1((16, 14), c, x0, y, eps=1e-9)
    assert rel_l2(out, ref0) < 5e-9


def test_no_bounded_wait_gave_up(native):
    n = ctypes.c_longlong(-1)
    assert native.gbn_wait_timeouts(ctypes.byref(n), 0) == 0
    assert n.value == 0
