"""The autotuner: its settings keep the accuracy of the defaults, its
choices are cached in memory and in the cache file, and the three ways of
using it (returned Opts, Opts(gpu_autotune=True), NufftBatch(autotune=True))
give the same transforms as the default settings."""
import os

import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def jf(native, tmp_path_factory):
    import jax_finufft_gb300

    path = tmp_path_factory.mktemp("tune") / "autotune.txt"
    old = os.environ.get("GBN_AUTOTUNE_CACHE")
    os.environ["GBN_AUTOTUNE_CACHE"] = str(path)
    from jax_finufft_gb300 import tune

    tune.clear_cache(forget_file=True)
    yield jax_finufft_gb300
    tune.clear_cache(forget_file=True)
    if old is None:
        del os.environ["GBN_AUTOTUNE_CACHE"]
    else:
        os.environ["GBN_AUTOTUNE_CACHE"] = old


def _points(rng, dim, M, rdt):
    return [torch.tensor(rng.uniform(-np.pi, np.pi, M).astype(rdt), device=DEV)
            for _ in range(dim)]


@pytest.mark.parametrize("ty, shape, M, single", [(1, (96, 80), 20000, True),
                                                  (2, (48, 40, 32), 30000, True),
                                                  (1, (300,), 5000, False)])
def test_tuned_settings_keep_accuracy(jf, ty, shape, M, single):
    from jax_finufft_gb300 import tune
    from oracle import direct

    rng = np.random.default_rng(5 + ty)
    cdt = torch.complex64 if single else torch.complex128
    rdt = np.float32 if single else np.float64
    eps = 1e-6 if single else 1e-9
    opts, info = tune.autotune(ty, shape, M, eps=eps, dtype=cdt)
    assert opts.gpu_upsampfac in (2.0, 1.25)
    assert opts.gpu_method in (0, 1, 2)
    assert not info["cached"]
    assert info["rel_err"] < 10 * eps
    _, info2 = tune.autotune(ty, shape, M, eps=eps, dtype=cdt)
    assert info2["cached"]
    x = _points(rng, len(shape), M, rdt)
    xs = [v.cpu().numpy().astype(np.float64) for v in x]
    if ty == 1:
        c = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), dtype=cdt,
                         device=DEV)
        tuned = jf.nufft1(shape, c, *x, eps=eps, opts=opts)
        plain = jf.nufft1(shape, c, *x, eps=eps)
        if M * np.prod(shape) <= 2e8:
            truth = direct.type1(c.cpu().numpy(), xs, shape, iflag=1)
            assert rel_l2(tuned.cpu().numpy(), truth) <= max(
                10 * eps, 1.5 * rel_l2(plain.cpu().numpy(), truth))
    else:
        f = torch.tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape),
                         dtype=cdt, device=DEV)
        tuned = jf.nufft2(f, *x, eps=eps, opts=opts)
        plain = jf.nufft2(f, *x, eps=eps)
    assert rel_l2(tuned.cpu().numpy(), plain.cpu().numpy()) < 20 * eps


def test_cache_file_and_reload(jf):
    from jax_finufft_gb300 import tune

    path = os.environ["GBN_AUTOTUNE_CACHE"]
    opts, info = tune.autotune(2, (64, 64), 10000, eps=1e-5)
    assert os.path.exists(path)
    with open(path) as fh:
        lines = [ln for ln in fh if "|" in ln]
    assert any("t2 d2 s1 n64x64x1" in ln for ln in lines)
    tune.clear_cache(forget_file=False)  # drop memory, reload from the file
    opts2, info2 = tune.autotune(2, (64, 64), 10000, eps=1e-5)
    assert info2["cached"]
    assert opts2 == opts


def test_opts_flag_matches_default(jf):
    from jax_finufft_gb300.options import Opts

    rng = np.random.default_rng(11)
    M, shape = 40000, (128, 128)
    x = _points(rng, 2, M, np.float32)
    f = torch.tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape),
                     dtype=torch.complex64, device=DEV)
    a = jf.nufft2(f, *x, eps=1e-6, opts=Opts(gpu_autotune=True))
    b = jf.nufft2(f, *x, eps=1e-6)
    assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 2e-5
    # differentiable path (fused forward keeps the tuned plan)
    fg = f.clone().requires_grad_(True)
    y = jf.nufft2(fg, *x, eps=1e-6, opts=Opts(gpu_autotune=True))
    (g,) = torch.autograd.grad(y.abs().square().sum(), fg)
    fh = f.clone().requires_grad_(True)
    y2 = jf.nufft2(fh, *x, eps=1e-6)
    (g2,) = torch.autograd.grad(y2.abs().square().sum(), fh)
    assert rel_l2(g.cpu().numpy(), g2.cpu().numpy()) < 5e-5


def test_batch_autotune_matches_single(jf):
    from jax_finufft_gb300.batch import NufftBatch

    rng = np.random.default_rng(12)
    shapes = [(64, 64), (128, 96), (64, 64), (40, 50)]
    Ms = [5000, 20000, 3000, 1000]
    pts = [tuple(rng.uniform(-np.pi, np.pi, M).astype(np.float32) for _ in range(2))
           for M in Ms]
    b = NufftBatch(2, shapes, Ms, eps=1e-6, autotune=True)
    src = [torch.tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s),
                        dtype=torch.complex64, device=DEV) for s in shapes]
    outs = b(pts, src)
    torch.cuda.synchronize()
    for k in range(len(Ms)):
        x = [torch.as_tensor(v, device=DEV) for v in pts[k]]
        ref = jf.nufft2(src[k], *x, eps=1e-6)
        assert rel_l2(outs[k].cpu().numpy(), ref.cpu().numpy()) < 2e-5, k
    assert b.info()["work_queue"]
