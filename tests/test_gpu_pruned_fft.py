"""Pruned 3D FFT (mode-region planes only) against the full cuFFT transform
and the FP64 direct sum, for type 1, type 2, the fused adjoint and type 3
(whose inner type 2 grid is pruned too)."""
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
    out = []
    for flag in ("0", "1"):
        old = os.environ.get("GBN_DISABLE_FFT_PRUNING")
        os.environ["GBN_DISABLE_FFT_PRUNING"] = flag
        try:
            r = fn()
            out.append(r.detach().clone() if torch.is_tensor(r) else [x.clone() for x in r])
        finally:
            if old is None:
                del os.environ["GBN_DISABLE_FFT_PRUNING"]
            else:
                os.environ["GBN_DISABLE_FFT_PRUNING"] = old
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("single", [True, False])
@pytest.mark.parametrize("shape", [(64, 64, 64), (70, 64, 66)])
def test_pruned_matches_full_and_direct(jf, single, shape):
    from oracle import direct

    rng = np.random.default_rng(17)
    M = 20000
    rdt = np.float32 if single else np.float64
    cdt = torch.complex64 if single else torch.complex128
    eps = 1e-6 if single else 1e-11
    xs = [rng.uniform(-np.pi, np.pi, M).astype(rdt) for _ in range(3)]
    x = [torch.tensor(v, device=DEV) for v in xs]
    c = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), dtype=cdt, device=DEV)
    f = torch.tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape), dtype=cdt,
                     device=DEV)
    tol = 1e-6 if single else 1e-13
    a1, b1 = _both(lambda: jf.nufft1(shape, c, *x, eps=eps))
    assert rel_l2(a1.cpu().numpy(), b1.cpu().numpy()) < tol
    a2, b2 = _both(lambda: jf.nufft2(f, *x, eps=eps))
    assert rel_l2(a2.cpu().numpy(), b2.cpu().numpy()) < tol
    # against the direct sums on subsets
    xd = [v.astype(np.float64) for v in xs]
    ks = [rng.integers(0, n, 40) for n in shape]
    fr = [direct.frequencies(n) for n in shape]
    sub = direct.type1(c.cpu().numpy(), xd, ks=[fr[a][ks[a]] for a in range(3)])
    got = a1.cpu().numpy()[np.ix_(ks[0], ks[1], ks[2])]
    assert rel_l2(got, sub) < (5 * max(eps, 1e-6) if single else 5 * eps)
    idx = rng.choice(M, 300, replace=False)
    tru = direct.type2(f.cpu().numpy(), [v[idx] for v in xd])
    assert rel_l2(a2.cpu().numpy()[idx], tru) < (5 * max(eps, 1e-6) if single else 5 * eps)


def test_pruned_fused_gradient(jf):
    rng = np.random.default_rng(18)
    M, shape = 20000, (64, 64, 64)
    x0 = [torch.tensor(rng.uniform(-np.pi, np.pi, M).astype(np.float32), device=DEV)
          for _ in range(3)]
    f0 = torch.tensor((rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
                      .astype(np.complex64), device=DEV)

    def grads():
        f = f0.clone().requires_grad_(True)
        x = [v.clone().requires_grad_(True) for v in x0]
        y = jf.nufft2(f, *x, eps=1e-6)
        return torch.autograd.grad(y.abs().square().sum(), [f] + x)

    a, b = _both(grads)
    for ga, gb in zip(a, b):
        assert rel_l2(ga.cpu().numpy(), gb.cpu().numpy()) < 2e-6


def test_pruned_type3(jf):
    rng = np.random.default_rng(19)
    M = N = 20000
    x = [torch.tensor(rng.uniform(-np.pi, np.pi, M), device=DEV) for _ in range(3)]
    s = [torch.tensor(rng.uniform(-40, 40, N), device=DEV) for _ in range(3)]
    c = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device=DEV)
    a, b = _both(lambda: jf.nufft3(c, *x, *s, eps=1e-9))
    assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-12
