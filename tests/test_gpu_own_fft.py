"""The library's pruned FP32 FFT for power-of-two fine grids (deconvolution
fused) against cuFFT with the separate deconvolution kernels
(GBN_DISABLE_OWN_FFT=1 at execute time), and against FP64 direct sums: every
dimension, both types, both mode orders, odd and even mode counts, stacked
transforms, FP64 data computed in FP32, and the adjoint execute of the fused
gradient."""
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


def _both(fn):
    """fn() with the library's FFT, then with cuFFT."""
    out = []
    for flag in ("0", "1"):
        old = os.environ.get("GBN_DISABLE_OWN_FFT")
        os.environ["GBN_DISABLE_OWN_FFT"] = flag
        try:
            r = fn()
            out.append(r.detach().clone())
        finally:
            if old is None:
                del os.environ["GBN_DISABLE_OWN_FFT"]
            else:
                os.environ["GBN_DISABLE_OWN_FFT"] = old
    torch.cuda.synchronize()
    return out


# shapes whose fine grids (sigma = 2) have 128, 256, 512 or 1024 cells per axis;
# odd mode counts (63, 127) exercise uneven mode regions
SHAPES = [(512,), (63,), (256, 128), (127, 64), (64, 64, 64), (63, 64, 128), (128, 64, 65)]


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("modeord", [0, 1])
def test_own_fft_matches_cufft_and_direct(jf, shape, modeord):
    from jax_finufft_gb300.options import Opts
    from oracle import direct

    ndim = len(shape)
    rng = np.random.default_rng(31 + 7 * ndim + modeord)
    M = 20000
    eps = 1e-6
    xs = [rng.uniform(-np.pi, np.pi, M).astype(np.float32) for _ in range(ndim)]
    x = [torch.tensor(v, device=DEV) for v in xs]
    ntr = 2
    c = torch.tensor((rng.standard_normal((ntr, M)) + 1j * rng.standard_normal((ntr, M)))
                     .astype(np.complex64), device=DEV)
    f = torch.tensor((rng.standard_normal((ntr,) + shape) + 1j * rng.standard_normal((ntr,) + shape))
                     .astype(np.complex64), device=DEV)
    opts = Opts(modeord=modeord)
    iflag = 1 if ndim % 2 else -1
    a1, b1 = _both(lambda: jf.nufft1(shape, c, *x, eps=eps, iflag=iflag, opts=opts))
    assert rel_l2(a1.cpu().numpy(), b1.cpu().numpy()) < 2e-6
    a2, b2 = _both(lambda: jf.nufft2(f, *x, eps=eps, iflag=-iflag, opts=opts))
    assert rel_l2(a2.cpu().numpy(), b2.cpu().numpy()) < 2e-6
    # direct sums on subsets (modes in the requested order)
    xd = [v.astype(np.float64) for v in xs]
    fr = [direct.frequencies(n, modeord) for n in shape]
    ks = [rng.integers(0, n, 24) for n in shape]
    sub = direct.type1(c[1].cpu().numpy(), xd, ks=[fr[a][ks[a]] for a in range(ndim)],
                       iflag=iflag)
    got = a1[1].cpu().numpy()[np.ix_(*ks)]
    assert rel_l2(got, sub) < 5e-6
    idx = rng.choice(M, 300, replace=False)
    tru = direct.type2(f[1].cpu().numpy(), [v[idx] for v in xd], iflag=-iflag, modeord=modeord)
    assert rel_l2(a2[1].cpu().numpy()[idx], tru) < 5e-6


def test_own_fft_fp64_data(jf):
    """complex128 data computed in FP32 (gpu_precision = 1)."""
    from jax_finufft_gb300.options import Opts

    rng = np.random.default_rng(41)
    M, shape = 10000, (64, 64, 64)
    x = [torch.tensor(rng.uniform(-np.pi, np.pi, M), device=DEV) for _ in range(3)]
    c = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device=DEV)
    f = torch.tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape), device=DEV)
    opts = Opts(gpu_precision=1)
    a1, b1 = _both(lambda: jf.nufft1(shape, c, *x, eps=1e-6, opts=opts))
    assert a1.dtype == torch.complex128
    assert rel_l2(a1.cpu().numpy(), b1.cpu().numpy()) < 2e-6
    a2, b2 = _both(lambda: jf.nufft2(f, *x, eps=1e-6, opts=opts))
    assert rel_l2(a2.cpu().numpy(), b2.cpu().numpy()) < 2e-6


def test_own_fft_fused_gradient(jf):
    """The fused adjoint runs the type-2 plan's adjoint (a type-1 execute) on
    the library's FFT too."""
    rng = np.random.default_rng(43)
    M, shape = 20000, (64, 64, 64)
    x0 = [torch.tensor(rng.uniform(-np.pi, np.pi, M).astype(np.float32), device=DEV)
          for _ in range(3)]
    f0 = torch.tensor((rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
                      .astype(np.complex64), device=DEV)
    y = torch.tensor((rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64),
                     device=DEV)

    def grad_f():
        f = f0.clone().requires_grad_(True)
        x = [v.clone().requires_grad_(True) for v in x0]
        loss = (jf.nufft2(f, *x, eps=1e-6) - y).abs().pow(2).sum()
        loss.backward()
        return torch.cat([f.grad.reshape(-1)] + [v.grad.to(torch.complex64) for v in x])

    a, b = _both(grad_f)
    assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-5
