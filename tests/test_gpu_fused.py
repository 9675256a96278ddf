"""The fused adjoint: gradients on the forward's sort, one batched FFT of the
stacked weighted grids and one interpolation pass.

Checked against the stacked-transform rules of the reference
(src/jax_finufft/ops.py:158-314, selected with gpu_fused_adjoint=False) and,
for the differentiated least-squares loss of the type-2 workload, against
central finite differences in float64 (32^3 modes, M=5,000, h=1e-6).
"""
from itertools import product

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


def _grads(jf, ty, args, opts, eps, iflag, shape=None):
    a = [t.detach().clone().requires_grad_(True) for t in args]
    if ty == 1:
        out = jf.nufft1(shape, a[0], *a[1:], eps=eps, iflag=iflag, opts=opts)
    else:
        out = jf.nufft2(a[0], *a[1:], eps=eps, iflag=iflag, opts=opts)
    w = torch.randn(out.shape, dtype=out.dtype, device=DEV, generator=torch.Generator(DEV).manual_seed(1))
    loss = torch.real(torch.sum(torch.conj(w) * out))
    return torch.autograd.grad(loss, a)


@pytest.mark.parametrize("ty, ndim, single", list(product([1, 2], [1, 2, 3], [True, False])))
def test_fused_matches_stacked(jf, ty, ndim, single):
    from jax_finufft_gb300.options import Opts

    rng = np.random.default_rng(40 + 10 * ty + ndim)
    rdt = torch.float32 if single else torch.float64
    cdt = torch.complex64 if single else torch.complex128
    eps = 1e-6 if single else 1e-11
    shape = {1: (64,), 2: (30, 24), 3: (14, 12, 16)}[ndim]
    M, T, B = 2000, 3, 2  # n_tot = B point sets, n_transf = T stacked transforms
    x = [torch.tensor(rng.uniform(-np.pi, np.pi, (B, 1, M)), dtype=rdt, device=DEV)
         for _ in range(ndim)]
    if ty == 1:
        src = torch.tensor(rng.normal(size=(B, T, M)) + 1j * rng.normal(size=(B, T, M)),
                           dtype=cdt, device=DEV)
    else:
        src = torch.tensor(rng.normal(size=(B, T) + shape) + 1j * rng.normal(size=(B, T) + shape),
                           dtype=cdt, device=DEV)
    for iflag in (-1, 1):
        g_f = _grads(jf, ty, [src] + x, Opts(gpu_fused_adjoint=True), eps, iflag, shape)
        g_s = _grads(jf, ty, [src] + x, Opts(gpu_fused_adjoint=False), eps, iflag, shape)
        tol = 2e-5 if single else 1e-9
        for a, b in zip(g_f, g_s):
            assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < tol


def test_least_squares_loss_finite_differences(jf):
    """L = sum_j |nufft2(c; x_j, y_j, z_j) - d_j|^2 in float64 at 32^3 modes and
    M=5000: dL/dc and dL/d(x, y, z) from the fused adjoint against central
    finite differences (h=1e-6) along random directions."""
    rng = np.random.default_rng(4)
    N, M = 32, 5000
    c = torch.tensor(rng.normal(size=(N, N, N)) + 1j * rng.normal(size=(N, N, N)),
                     device=DEV)
    c2 = torch.tensor(rng.normal(size=(N, N, N)) + 1j * rng.normal(size=(N, N, N)),
                      device=DEV)
    pts = [torch.tensor(rng.uniform(-np.pi, np.pi, M), device=DEV) for _ in range(3)]
    d = jf.nufft2(c2, *pts, eps=1e-12) + 0.1 * torch.tensor(
        rng.normal(size=M) + 1j * rng.normal(size=M), device=DEV)

    def loss(cc, *p):
        r = jf.nufft2(cc, *p, eps=1e-12) - d
        return torch.sum(torch.real(r) ** 2 + torch.imag(r) ** 2)

    a = [c.clone().requires_grad_(True)] + [p.clone().requires_grad_(True) for p in pts]
    grads = torch.autograd.grad(loss(*a), a)
    h = 1e-6
    for trial in range(3):
        dirs = [torch.tensor(rng.normal(size=c.shape) + 1j * rng.normal(size=c.shape),
                             device=DEV)] + [torch.tensor(rng.normal(size=M), device=DEV)
                                             for _ in range(3)]
        with torch.no_grad():
            lp = loss(*[v + h * dv for v, dv in zip([c] + pts, dirs)])
            lm = loss(*[v - h * dv for v, dv in zip([c] + pts, dirs)])
        fd = float((lp - lm) / (2 * h))
        # torch's gradient of a real loss w.r.t. a complex input is dL/dRe + i dL/dIm
        an = float(torch.sum(torch.real(torch.conj(grads[0]) * dirs[0])))
        an += sum(float(torch.sum(gp * dp)) for gp, dp in zip(grads[1:], dirs[1:]))
        assert abs(fd - an) <= 1e-6 * max(abs(fd), 1.0), (fd, an)


def test_fused_path_sorts_once(jf):
    """Forward + backward of a type-2 transform with all gradients: the fused
    adjoint sorts the points once (the forward's), the stacked rules sort in
    each of their transforms."""
    from jax_finufft_gb300 import _native
    from jax_finufft_gb300.options import Opts

    lib = _native.load()
    rng = np.random.default_rng(9)
    f = torch.tensor(rng.normal(size=(24, 20, 16)) + 1j * rng.normal(size=(24, 20, 16)),
                     dtype=torch.complex64, device=DEV)
    x = [torch.tensor(rng.uniform(-np.pi, np.pi, 4000), dtype=torch.float32, device=DEV)
         for _ in range(3)]

    def launches(opts):
        a = [f.clone().requires_grad_(True)] + [p.clone().requires_grad_(True) for p in x]
        torch.cuda.synchronize()
        n0 = lib.gbn_launch_count()
        out = jf.nufft2(a[0], *a[1:], eps=1e-5, opts=opts)
        torch.autograd.grad(torch.sum(torch.abs(out) ** 2), a)
        torch.cuda.synchronize()
        return lib.gbn_launch_count() - n0

    fused = launches(Opts(gpu_fused_adjoint=True))
    stacked = launches(Opts(gpu_fused_adjoint=False))
    assert fused < stacked


def _grads3(jf, args, ndim, opts, eps, iflag):
    a = [t.detach().clone().requires_grad_(i <= ndim) for i, t in enumerate(args)]
    out = jf.nufft3(a[0], *a[1:], eps=eps, iflag=iflag, opts=opts)
    w = torch.randn(out.shape, dtype=out.dtype, device=DEV,
                    generator=torch.Generator(DEV).manual_seed(3))
    loss = torch.real(torch.sum(torch.conj(w) * out))
    return torch.autograd.grad(loss, a[:ndim + 1])


@pytest.mark.parametrize("ndim, single", list(product([1, 2, 3], [True, False])))
def test_fused_type3_matches_stacked(jf, ndim, single):
    """Type-3 strength and source gradients from one adjoint pass on the
    forward's plans against the stacked rules (ops.py:238-260, 280-314).
    The source gradients differentiate the adjoint's interpolant, whose
    aliasing error the derivative amplifies by about the ratio of the grid
    frequency to the signal's: they agree to a few times eps."""
    from jax_finufft_gb300.options import Opts

    rng = np.random.default_rng(70 + ndim)
    rdt = torch.float32 if single else torch.float64
    cdt = torch.complex64 if single else torch.complex128
    eps = 1e-6 if single else 1e-11
    M, Nt, T, B = 3000, 800, 2, 2
    x = [torch.tensor(rng.uniform(-np.pi, np.pi, (B, 1, M)), dtype=rdt, device=DEV)
         for _ in range(ndim)]
    s = [torch.tensor(rng.uniform(-25, 25, (B, 1, Nt)), dtype=rdt, device=DEV)
         for _ in range(ndim)]
    c = torch.tensor(rng.normal(size=(B, T, M)) + 1j * rng.normal(size=(B, T, M)), dtype=cdt,
                     device=DEV)
    for iflag in (-1, 1):
        g_f = _grads3(jf, [c] + x + s, ndim, Opts(gpu_fused_adjoint=True), eps, iflag)
        g_s = _grads3(jf, [c] + x + s, ndim, Opts(gpu_fused_adjoint=False), eps, iflag)
        assert rel_l2(g_f[0].cpu().numpy(), g_s[0].cpu().numpy()) < (2e-5 if single else 1e-9)
        for a, b in zip(g_f[1:], g_s[1:]):
            assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < (1e-4 if single else 1e-8)


def test_fused_type3_finite_differences(jf):
    """Float64 type-3 loss sum |nufft3(c; x) - d|^2 (3D): the fused strength
    and source gradients against central finite differences (h = 1e-6) along
    random directions."""
    rng = np.random.default_rng(77)
    M, Nt = 600, 300
    x0 = [rng.uniform(-np.pi, np.pi, M) for _ in range(3)]
    s = [torch.tensor(rng.uniform(-12, 12, Nt), device=DEV) for _ in range(3)]
    c0 = rng.normal(size=M) + 1j * rng.normal(size=M)
    d = torch.tensor(rng.normal(size=Nt) + 1j * rng.normal(size=Nt), device=DEV)

    def loss(c, xs):
        r = jf.nufft3(c, *xs, *s, eps=1e-12, iflag=1) - d
        return torch.sum(torch.real(r) ** 2 + torch.imag(r) ** 2)

    c = torch.tensor(c0, device=DEV, requires_grad=True)
    xs = [torch.tensor(v, device=DEV, requires_grad=True) for v in x0]
    grads = torch.autograd.grad(loss(c, xs), [c] + xs)
    h = 1e-6
    for k in range(4):
        dc = rng.normal(size=M) + 1j * rng.normal(size=M)
        dx = [rng.normal(size=M) for _ in range(3)]
        with torch.no_grad():
            lp = loss(torch.tensor(c0 + h * dc, device=DEV),
                      [torch.tensor(v + h * e, device=DEV) for v, e in zip(x0, dx)])
            lm = loss(torch.tensor(c0 - h * dc, device=DEV),
                      [torch.tensor(v - h * e, device=DEV) for v, e in zip(x0, dx)])
        fd = float((lp - lm) / (2 * h))
        an = float(torch.sum(torch.real(torch.conj(grads[0]) * torch.tensor(dc, device=DEV))))
        an += sum(float(torch.sum(gx * torch.tensor(e, device=DEV))) for gx, e in zip(grads[1:], dx))
        assert abs(an - fd) <= 1e-6 * max(1.0, abs(fd)), (k, an, fd)
