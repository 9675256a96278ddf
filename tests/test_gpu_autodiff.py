"""Gradients, forward-mode derivatives and vmap on the GPU path.

Mirrors tests/ops_test.py:128-377 and 400-491 of the reference: derivative
rules checked against central finite differences (torch.autograd.gradcheck,
reverse and forward mode) in float64 at eps=1e-12, per-argument gradients
consistent with joint ones, and vmap equal to a Python loop for mapped and
unmapped sources/points.
"""
from functools import partial
from itertools import product

import numpy as np
import pytest
import torch

from helpers import check_close

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def jf(native):
    import jax_finufft_gb300

    return jax_finufft_gb300


def _rand(rng, shape, lo=-np.pi, hi=np.pi):
    return torch.tensor(rng.uniform(lo, hi, size=shape), device=DEV, dtype=torch.float64)


def _crand(rng, shape):
    return torch.tensor(rng.normal(size=shape) + 1j * rng.normal(size=shape), device=DEV,
                        dtype=torch.complex128)


GRAD = list(product([1, 2, 3], [-1, 1]))


def _gradcheck(fn, args):
    args = tuple(a.detach().requires_grad_(True) for a in args)
    # spreading accumulates with atomics, so repeated backward passes differ
    # in the last bits: allow that nondeterminism, as for any atomic kernel
    assert torch.autograd.gradcheck(fn, args, eps=1e-6, atol=1e-5, rtol=1e-4,
                                    nondet_tol=1e-9, check_forward_ad=True,
                                    check_batched_grad=False, fast_mode=True)


@pytest.mark.parametrize("ndim, iflag", GRAD)
def test_nufft1_grad(jf, ndim, iflag):
    rng = np.random.default_rng(657)
    nu = tuple(int(v) for v in 12 // ndim + 3 * np.arange(ndim))
    x = [_rand(rng, 20) for _ in range(ndim)]
    c = _crand(rng, 20)
    fn = partial(jf.nufft1, nu, eps=1e-12, iflag=iflag)
    _gradcheck(fn, (c, *x))


@pytest.mark.parametrize("ndim, iflag", GRAD)
def test_nufft2_grad(jf, ndim, iflag):
    rng = np.random.default_rng(657)
    nu = tuple(int(v) for v in 12 // ndim + 3 * np.arange(ndim))
    x = [_rand(rng, 20) for _ in range(ndim)]
    f = _crand(rng, nu)
    fn = partial(jf.nufft2, eps=1e-12, iflag=iflag)
    _gradcheck(fn, (f, *x))


@pytest.mark.parametrize("ndim, iflag", GRAD)
def test_nufft3_grad(jf, ndim, iflag):
    rng = np.random.default_rng(657)
    x = [_rand(rng, 15, -1.0, 1.0) for _ in range(ndim)]
    s = [_rand(rng, 12, -1.0, 1.0) for _ in range(ndim)]
    c = _crand(rng, 15)
    fn = partial(jf.nufft3, eps=1e-12, iflag=iflag)
    _gradcheck(fn, (c, *x, *s))


@pytest.mark.parametrize("ty", [1, 2, 3])
def test_grad_argnum_consistency(jf, ty):
    """Gradients taken one argument at a time equal the joint gradient
    (ops_test.py:152-157)."""
    rng = np.random.default_rng(3)
    ndim = 2
    if ty == 1:
        args = [_crand(rng, 30)] + [_rand(rng, 30) for _ in range(ndim)]
        fn = partial(jf.nufft1, (11, 9), eps=1e-12)
    elif ty == 2:
        args = [_crand(rng, (11, 9))] + [_rand(rng, 30) for _ in range(ndim)]
        fn = partial(jf.nufft2, eps=1e-12)
    else:
        args = [_crand(rng, 30)] + [_rand(rng, 30) for _ in range(2 * ndim)]
        fn = partial(jf.nufft3, eps=1e-12)

    def scalar(*a):
        return torch.linalg.norm(fn(*a))

    joint = torch.autograd.grad(scalar(*[a.requires_grad_(True) for a in args]), args)
    for n in range(len(args)):
        a = [t.detach().requires_grad_(i == n) for i, t in enumerate(args)]
        (g,) = torch.autograd.grad(scalar(*a), [a[n]])
        check_close(g.cpu().numpy(), joint[n].detach().cpu().numpy())


@pytest.mark.parametrize("ndim, iflag", GRAD)
def test_nufft1_vmap(jf, ndim, iflag):
    rng = np.random.default_rng(657)
    R = 5
    nu = tuple(int(v) for v in 35 // ndim + 5 * np.arange(ndim))
    x = [_rand(rng, (R, 50)) for _ in range(ndim)]
    c = _crand(rng, (R, 50))
    func = partial(jf.nufft1, nu, iflag=iflag)
    calc = torch.func.vmap(func)(c, *x)
    for n in range(R):
        check_close(calc[n].cpu().numpy(), func(c[n], *(v[n] for v in x)).cpu().numpy())
    calc_ax = torch.func.vmap(func, in_dims=(1,) + (0,) * ndim)(c.movedim(0, 1).contiguous(), *x)
    check_close(calc_ax.cpu().numpy(), calc.cpu().numpy())
    calc_unmap = torch.func.vmap(func, in_dims=(None,) + (0,) * ndim)(c[0], *x)
    for n in range(R):
        check_close(calc_unmap[n].cpu().numpy(), func(c[0], *(v[n] for v in x)).cpu().numpy())
    calc_pt = torch.func.vmap(func, in_dims=(0,) + (0,) * (ndim - 1) + (None,))(
        c, *x[:-1], x[-1][0])
    for n in range(R):
        check_close(calc_pt[n].cpu().numpy(),
                    func(c[n], *(v[n] for v in x[:-1]), x[-1][0]).cpu().numpy())


@pytest.mark.parametrize("ndim, iflag", GRAD)
def test_nufft2_vmap(jf, ndim, iflag):
    rng = np.random.default_rng(657)
    R = 5
    nu = tuple(int(v) for v in 35 // ndim + 5 * np.arange(ndim))
    x = [_rand(rng, (R, 50)) for _ in range(ndim)]
    f = _crand(rng, (R,) + nu)
    func = partial(jf.nufft2, iflag=iflag)
    calc = torch.func.vmap(func)(f, *x)
    for n in range(R):
        check_close(calc[n].cpu().numpy(), func(f[n], *(v[n] for v in x)).cpu().numpy())
    calc_unmap = torch.func.vmap(func, in_dims=(None,) + (0,) * ndim)(f[0], *x)
    for n in range(R):
        check_close(calc_unmap[n].cpu().numpy(), func(f[0], *(v[n] for v in x)).cpu().numpy())
    calc_pt = torch.func.vmap(func, in_dims=(0,) + (0,) * (ndim - 1) + (None,))(
        f, *x[:-1], x[-1][0])
    for n in range(R):
        check_close(calc_pt[n].cpu().numpy(),
                    func(f[n], *(v[n] for v in x[:-1]), x[-1][0]).cpu().numpy())


@pytest.mark.parametrize("ndim, iflag", GRAD)
def test_nufft3_vmap(jf, ndim, iflag):
    rng = np.random.default_rng(657)
    R = 5
    x = [_rand(rng, (R, 50)) for _ in range(ndim)]
    s = [_rand(rng, (R, 35), -1.0, 1.0) for _ in range(ndim)]
    c = _crand(rng, (R, 50))
    func = partial(jf.nufft3, iflag=iflag)
    calc = torch.func.vmap(func)(c, *x, *s)
    for n in range(R):
        check_close(calc[n].cpu().numpy(),
                    func(c[n], *(v[n] for v in x), *(v[n] for v in s)).cpu().numpy())
    calc_unmap = torch.func.vmap(func, in_dims=(None,) + (0,) * 2 * ndim)(c[0], *x, *s)
    for n in range(R):
        check_close(calc_unmap[n].cpu().numpy(),
                    func(c[0], *(v[n] for v in x), *(v[n] for v in s)).cpu().numpy())


def test_vmap_grad_shapes(jf):
    """gh54 regression (ops_test.py:454-491): jvp/grad shapes under vmap with
    N(0,1) points, i.e. points outside one period."""
    rng = np.random.default_rng(54)
    f = _crand(rng, (8, 1000))
    x = torch.tensor(rng.normal(size=(8, 3, 1000)), device=DEV)

    def aux(f1, x1):
        return torch.real(jf.nufft1((16, 16, 16), f1, *x1, iflag=-1)).mean()

    def test(f, x):
        return torch.func.vmap(aux)(f, x).mean()

    gx = torch.func.grad(test, argnums=1)(f, x)
    assert gx.shape == x.shape
    gf = torch.func.grad(test, argnums=0)(f, x)
    assert gf.shape == f.shape
    val, tan = torch.func.jvp(lambda xx: test(f, xx), (x,), (torch.ones_like(x),))
    assert val.shape == tan.shape == ()

    g2 = _crand(rng, (8, 16, 16, 16))

    def aux2(f1, x1):
        return torch.real(jf.nufft2(f1, *x1, iflag=-1)).mean()

    gx2 = torch.func.grad(lambda xx: torch.func.vmap(aux2)(g2, xx).mean())(x)
    assert gx2.shape == x.shape
