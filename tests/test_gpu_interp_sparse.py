"""Type-2 interpolation of sparse and dense subproblems in one transform.

Each case mixes a sparse spread of points (subproblems of one to a few
points, each staging a whole tile; points whose support wraps around the
grid) with a dense cluster (full subproblems) and compares the library with
the FP64 oracle (oracle/cpu_nufft.py) in relative l2 within 5 max(eps, 1e-6)
(complex64) or 5 eps (complex128), the bound of the other GPU parity tests.
The same kind of points through a batched plan (the work-queue
interpolation, problems from 40 to 50,000 points) are compared with one
plain call per problem.
"""
import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _points(seed, dim, n_sparse, n_dense):
    rng = np.random.default_rng(seed)
    x = []
    for _ in range(dim):
        sparse = rng.uniform(-np.pi, np.pi, n_sparse)
        sparse[:4] = [-np.pi, np.pi - 1e-6, -3.14, 3.1]  # supports that wrap
        x.append(np.concatenate([sparse, rng.normal(0.5, 0.05, n_dense)]))
    return x


@pytest.mark.parametrize("dim,shape", [(2, (96, 80)), (3, (40, 36, 32))])
@pytest.mark.parametrize("dtype,eps", [(np.complex64, 1e-5), (np.complex128, 1e-9)])
def test_sparse_and_dense_subproblems_match_oracle(dim, shape, dtype, eps):
    import jax_finufft_gb300 as jf
    from oracle import cpu_nufft as cn

    rng = np.random.default_rng(3 + dim)
    x = _points(11 + dim, dim, 300, 20000)
    f = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(dtype)
    rdt = np.float32 if dtype == np.complex64 else np.float64
    xt = [torch.tensor(v.astype(rdt), device="cuda") for v in x]
    out = jf.nufft2(torch.tensor(f, device="cuda"), *xt, eps=eps, iflag=-1).cpu().numpy()
    ref = cn.nufft2(f.astype(np.complex128), *[v.astype(rdt).astype(np.float64) for v in x],
                    eps=eps, iflag=-1)
    bound = 5 * max(eps, 1e-6) if dtype == np.complex64 else 5 * eps
    assert np.isfinite(out).all()
    assert rel_l2(out, ref) < bound, rel_l2(out, ref)
    # the sparse points alone (every subproblem gathers directly)
    n = 300
    out_s = jf.nufft2(torch.tensor(f, device="cuda"), *[v[:n] for v in xt], eps=eps,
                      iflag=-1).cpu().numpy()
    assert rel_l2(out_s, ref[:n]) < bound, rel_l2(out_s, ref[:n])


def test_sparse_problems_in_a_batch_match_single_calls():
    """A type-2 batch of problems from very sparse to dense (the work-queue
    kernel's subproblems take both paths) against one plain call each."""
    import jax_finufft_gb300 as jf
    from jax_finufft_gb300.batch import NufftBatch

    rng = np.random.default_rng(8)
    shapes = [(128, 128), (64, 96), (256, 256), (128, 128)]
    Ms = [40, 3000, 200, 50000]
    pts = [[torch.tensor(rng.uniform(-np.pi, np.pi, m).astype(np.float32), device="cuda")
            for _ in range(2)] for m in Ms]
    fs = [torch.tensor((rng.normal(size=s) + 1j * rng.normal(size=s)).astype(np.complex64),
                       device="cuda") for s in shapes]
    b = NufftBatch(2, shapes, Ms, eps=1e-6, use_graph=False)
    c = b.empty_strengths()
    b.run_packed(b.pack_points(pts), c, torch.cat([f.reshape(-1) for f in fs]))
    torch.cuda.synchronize()
    for k in range(len(Ms)):
        one = jf.nufft2(fs[k], *pts[k], eps=1e-6).cpu().numpy()
        got = c[int(b.pt_off[k]):int(b.pt_off[k + 1])].cpu().numpy()
        assert rel_l2(got, one) < 1e-5, (k, rel_l2(got, one))
