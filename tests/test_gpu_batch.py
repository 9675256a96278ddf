"""Batched plans against the single-problem path.

K independent problems of different point counts and mode shapes (and a
per-problem upsampling factor) run as one batch -- per-problem sorting and
deconvolution, grouped cuFFT, one persistent work-queue kernel -- and every
problem's output must match the same transform through nufft1/nufft2.  The
graph-captured form must give the same results on replay, including after
the point values change in place.
"""
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


def _problems(rng, dim, K, single):
    rdt = np.float32 if single else np.float64
    shapes, Ms, pts = [], [], []
    choices = {1: [(64,), (128,), (200,)], 2: [(32, 32), (64, 48), (40, 40)],
               3: [(16, 16, 16), (20, 12, 24)]}[dim]
    for k in range(K):
        shapes.append(choices[k % len(choices)])
        M = int(10 ** rng.uniform(2, 4)) if k != 3 else 0  # one empty problem
        Ms.append(M)
        pts.append(tuple(rng.uniform(-np.pi, np.pi, M).astype(rdt) for _ in range(dim)))
    return shapes, Ms, pts


def _truth(ty, src_k, pts_k, shape, T):
    """FP64 direct sums for one problem, (T, ...) stacked."""
    from oracle import direct

    x = [np.asarray(v, dtype=np.float64) for v in pts_k]
    s = src_k.cpu().numpy().reshape((T, -1) if ty == 1 else (T,) + shape)
    if ty == 1:
        return np.stack([direct.type1(s[t], x, shape, iflag=1) for t in range(T)])
    return np.stack([direct.type2(s[t], x, iflag=-1) for t in range(T)])


@pytest.mark.parametrize("ty, dim, single, T", [(1, 2, True, 1), (2, 2, True, 1),
                                                (2, 1, False, 2), (1, 3, True, 3),
                                                (2, 3, False, 1), (1, 1, True, 2)])
def test_batch_matches_single(jf, ty, dim, single, T):
    """Every problem of the batch agrees with nufft1/nufft2 on the same
    problem.  Problems alternate sigma = 2 and 1.25; at 1.25 in FP32 the
    deconvolution amplifies FFT round-off so both paths sit near 5e-5 of the
    direct sum, and the agreement asked for is then three times the single
    path's own error against that sum (at sigma = 2, the plain tolerance)."""
    from jax_finufft_gb300.batch import NufftBatch
    from jax_finufft_gb300.options import Opts

    rng = np.random.default_rng(20 + 10 * ty + dim)
    K = 7
    shapes, Ms, pts = _problems(rng, dim, K, single)
    cdt = torch.complex64 if single else torch.complex128
    eps = 1e-6 if single else 1e-10
    tol = 1e-5 if single else 1e-9
    sig = [2.0 if k % 2 == 0 else 1.25 for k in range(K)]
    for use_graph in (False, True):
        b = NufftBatch(ty, shapes, Ms, ntransf=T, eps=eps, dtype=cdt, upsampfac=sig,
                       use_graph=use_graph)
        if ty == 1:
            src = [torch.tensor(rng.normal(size=(T, M)) + 1j * rng.normal(size=(T, M)),
                                dtype=cdt, device=DEV) for M in Ms]
        else:
            src = [torch.tensor(rng.normal(size=(T,) + s) + 1j * rng.normal(size=(T,) + s),
                                dtype=cdt, device=DEV) for s in shapes]
        refs, tols = [], []
        for k in range(K):
            x = [torch.as_tensor(v, device=DEV) for v in pts[k]]
            s_k = src[k] if T > 1 else src[k][0]
            o = Opts(gpu_upsampfac=sig[k])
            if ty == 1:
                ref = jf.nufft1(shapes[k], s_k, *x, eps=eps, opts=o)
            else:
                ref = jf.nufft2(s_k, *x, eps=eps, opts=o)
            refs.append(ref)
            if Ms[k] == 0:
                tols.append(None)
                continue
            tru = _truth(ty, src[k], pts[k], shapes[k], T)
            own = rel_l2(ref.cpu().numpy().reshape(tru.shape), tru)
            tols.append(max(tol, 3 * own) if sig[k] != 2.0 else tol)
        for rep in range(2):
            outs = b(pts, src)
            torch.cuda.synchronize()
            for k in range(K):
                if Ms[k] == 0:
                    if ty == 1:
                        assert torch.count_nonzero(outs[k]) == 0
                    continue
                err = rel_l2(outs[k].cpu().numpy(), refs[k].cpu().numpy())
                assert err < tols[k], (k, rep, use_graph, err, tols[k])


def test_graph_replay_follows_new_points(jf):
    """The captured graph reads the packed buffers at replay: changing the
    point values in place changes the result like a fresh call."""
    from jax_finufft_gb300.batch import NufftBatch

    rng = np.random.default_rng(3)
    shapes = [(48, 40), (64, 64), (48, 40)]
    Ms = [3000, 5000, 1000]
    b = NufftBatch(2, shapes, Ms, eps=1e-6, use_graph=True)
    P = b.empty_points()
    f = b.empty_modes()
    c = b.empty_strengths()
    f.copy_(torch.tensor((rng.normal(size=f.numel()) + 1j * rng.normal(size=f.numel()))
                         .astype(np.complex64), device=DEV))
    results = []
    for trial in range(3):
        P.copy_(torch.tensor(rng.uniform(-np.pi, np.pi, P.shape).astype(np.float32),
                             device=DEV))
        b.run_packed(P, c, f)
        torch.cuda.synchronize()
        for k in range(3):
            x = [P[u, b.pt_off[k]:b.pt_off[k + 1]] for u in range(2)]
            fk = f[b.mode_off[k]:b.mode_off[k + 1]].reshape(shapes[k])
            ref = jf.nufft2(fk, *x, eps=1e-6)
            got = c[b.pt_off[k]:b.pt_off[k + 1]]
            assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) < 1e-5
        results.append(c.clone())
    assert not torch.equal(results[0], results[1])
    assert b.info()["work_queue"]


def test_chain_of_type1_and_type2_batches(jf):
    """A chain runs a type-1 batch (one problem, stacked transforms: the
    plain per-subproblem kernels) and a type-2 batch (several problems: the
    work queue) as one pass; captured and replayed, twice, it gives each
    batch's own results, and the replay follows point values changed in
    place."""
    from jax_finufft_gb300.batch import NufftBatch, NufftBatchChain

    rng = np.random.default_rng(42)
    T, M1 = 4, 20000
    b1 = NufftBatch(1, [(64, 64)], [M1], ntransf=T, eps=1e-6, use_graph=False)
    shapes = [(32, 32), (64, 48), (40, 40)]
    Ms = [3000, 500, 8000]
    b2 = NufftBatch(2, shapes, Ms, eps=1e-6, use_graph=False)
    P1 = b1.pack_points([tuple(rng.uniform(-np.pi, np.pi, M1).astype(np.float32)
                               for _ in range(2))])
    c1 = torch.tensor((rng.standard_normal(T * M1) + 1j * rng.standard_normal(T * M1))
                      .astype(np.complex64), device=DEV)
    P2 = b2.pack_points([tuple(rng.uniform(-np.pi, np.pi, m).astype(np.float32)
                               for _ in range(2)) for m in Ms])
    f2 = torch.tensor((rng.standard_normal(sum(int(np.prod(s)) for s in shapes)) +
                       1j * rng.standard_normal(sum(int(np.prod(s)) for s in shapes)))
                      .astype(np.complex64), device=DEV)
    f1_ref, c2_ref = b1.empty_modes(), b2.empty_strengths()
    b1.run_packed(P1, c1, f1_ref)
    b2.run_packed(P2, c2_ref, f2)
    # the single problem matches nufft1 on the same data
    plain = jf.nufft1((64, 64), c1.reshape(T, M1), P1[0], P1[1], eps=1e-6)
    assert rel_l2(f1_ref.reshape(T, 64, 64).cpu().numpy(), plain.cpu().numpy()) < 1e-5
    chain = NufftBatchChain([b1, b2], use_graph=True)
    f1, c2 = b1.empty_modes(), b2.empty_strengths()
    for _ in range(2):
        f1.zero_()
        c2.zero_()
        chain.run_packed([(P1, c1, f1), (P2, c2, f2)])
        torch.cuda.synchronize()
        assert rel_l2(f1.cpu().numpy(), f1_ref.cpu().numpy()) < 1e-5
        assert rel_l2(c2.cpu().numpy(), c2_ref.cpu().numpy()) < 1e-5
    # new point values at the same addresses: the replayed graph re-sorts them
    P1.copy_(torch.remainder(P1 + 0.37, 2 * np.pi) - np.pi)
    P2.copy_(torch.remainder(P2 - 0.11, 2 * np.pi) - np.pi)
    b1.run_packed(P1, c1, f1_ref)
    b2.run_packed(P2, c2_ref, f2)
    chain.run_packed([(P1, c1, f1), (P2, c2, f2)])
    torch.cuda.synchronize()
    assert rel_l2(f1.cpu().numpy(), f1_ref.cpu().numpy()) < 1e-5
    assert rel_l2(c2.cpu().numpy(), c2_ref.cpu().numpy()) < 1e-5
    del chain
