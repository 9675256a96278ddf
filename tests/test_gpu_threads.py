"""Concurrent calls from a thread pool (the reference's
tests/freethreaded_test.py): ctypes releases the GIL around every library
call, so threads really do enter the library at the same time, on the
one-shot path (plans taken from the library's cache one caller at a time)
and on the fused path (Python plan cache with a lock per plan).  Results
must match the same transforms run one after another."""
import concurrent.futures

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


def test_threaded_pool_nufft1(jf, n_transforms=200, n_points=1000):
    rng = np.random.default_rng(42)
    modes = 64
    x = torch.tensor(rng.uniform(-np.pi, np.pi, (n_transforms, n_points)).astype(np.float32),
                     device=DEV)
    c = torch.tensor((rng.normal(size=(n_transforms, n_points))
                      + 1j * rng.normal(size=(n_transforms, n_points))).astype(np.complex64),
                     device=DEV)

    def compute(i):
        out = jf.nufft1(modes, c[i], x[i], eps=1e-6)
        torch.cuda.current_stream().synchronize()
        return out.cpu().numpy()

    sequential = [compute(i) for i in range(n_transforms)]
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        parallel = list(ex.map(compute, range(n_transforms)))
    for a, b in zip(sequential, parallel):
        assert rel_l2(b, a) < 1e-6


def test_threaded_fused_gradients(jf, n_jobs=32):
    rng = np.random.default_rng(43)
    shape, M = (24, 20, 16), 3000
    fs = [torch.tensor((rng.normal(size=shape) + 1j * rng.normal(size=shape))
                       .astype(np.complex64), device=DEV) for _ in range(n_jobs)]
    xs = [[torch.tensor(rng.uniform(-np.pi, np.pi, M).astype(np.float32), device=DEV)
           for _ in range(3)] for _ in range(n_jobs)]

    def grads(i):
        f = fs[i].clone().requires_grad_(True)
        x = [v.clone().requires_grad_(True) for v in xs[i]]
        y = jf.nufft2(f, *x, eps=1e-6)
        g = torch.autograd.grad(y.abs().square().sum(), [f] + x)
        torch.cuda.current_stream().synchronize()
        return [t.cpu().numpy() for t in g]

    sequential = [grads(i) for i in range(n_jobs)]
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        parallel = list(ex.map(grads, range(n_jobs)))
    for a, b in zip(sequential, parallel):
        for ga, gb in zip(a, b):
            assert rel_l2(gb, ga) < 1e-5
