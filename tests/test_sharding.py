"""The data-parallel patterns of jax_finufft_gb300.sharding on two gloo ranks.

Mirrors the reference's tests/sharding_test.py:70-334 on CPU processes: each
pattern's sharded value and gradient must equal the single-process result.
The per-rank transform is test infrastructure on CPU tensors:
  * forward values: the oracle port (oracle/cpu_nufft.py, the CPU
    restatement of the fast algorithm, FP64, eps 1e-10);
  * values and gradients: an FP64 direct NUDFT written with torch
    operations, so autograd differentiates it (the known answer the
    reference's tests compute, tests/ops_test.py:42-45, 77-84, 112-116).
Tolerance: the reference's check_close rtol for float64/complex128 (1e-7).
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WS = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _freqs(n):
    return torch.arange(-(n // 2), (n + 1) // 2, dtype=torch.float64)


def direct1(output_shape, c, *x, iflag=1, eps=None):
    ks = torch.meshgrid(*[_freqs(n) for n in output_shape], indexing="ij")
    ph = sum(k.reshape(-1, 1) * xi.reshape(1, -1) for k, xi in zip(ks, x))
    return (torch.exp(1j * iflag * ph) @ c).reshape(output_shape)


def direct2(f, *x, iflag=-1, eps=None):
    ks = torch.meshgrid(*[_freqs(n) for n in f.shape], indexing="ij")
    ph = sum(xi.reshape(-1, 1) * k.reshape(1, -1) for k, xi in zip(ks, x))
    return torch.exp(1j * iflag * ph) @ f.reshape(-1)


def direct3(c, *pts, iflag=-1, eps=None):
    d = len(pts) // 2
    ph = sum(pts[d + a].reshape(-1, 1) * pts[a].reshape(1, -1) for a in range(d))
    return torch.exp(1j * iflag * ph) @ c


def oracle_transform(kind):
    """The oracle port as a per-rank transform on CPU tensors (forward only)."""
    sys.path.insert(0, REPO)
    from oracle import cpu_nufft

    def t1(shape, c, *x, iflag=1, eps=1e-10):
        return torch.from_numpy(cpu_nufft.nufft1(shape, c.numpy(), *[v.numpy() for v in x],
                                                 eps=eps, iflag=iflag))

    def t2(f, *x, iflag=-1, eps=1e-10):
        return torch.from_numpy(cpu_nufft.nufft2(f.detach().numpy(), *[v.numpy() for v in x],
                                                 eps=eps, iflag=iflag))

    def t3(c, *pts, iflag=-1, eps=1e-10):
        return torch.from_numpy(cpu_nufft.nufft3(c.detach().numpy(),
                                                 *[v.detach().numpy() for v in pts],
                                                 eps=eps, iflag=iflag))

    return {1: t1, 2: t2, 3: t3}[kind]


def _inputs(ndim, ws):
    """The draws of sharding_test.py (seed 657, 32 points per device)."""
    rng = np.random.default_rng(657)
    n = 32 * ws
    nu = tuple(int(v) for v in 4 + np.arange(ndim))
    x = [rng.uniform(-np.pi, np.pi, n) for _ in range(ndim)]
    grid = rng.normal(size=nu) + 1j * rng.normal(size=nu)
    data = rng.normal(size=n) + 1j * rng.normal(size=n)
    src = [rng.uniform(-1.0, 1.0, n) for _ in range(ndim)]
    tgt = [rng.uniform(-1.0, 1.0, 20) for _ in range(ndim)]
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    tdat = rng.normal(size=20) + 1j * rng.normal(size=20)
    tgt_s = [rng.uniform(-1.0, 1.0, n) for _ in range(ndim)]
    src_r = [rng.uniform(-1.0, 1.0, 20) for _ in range(ndim)]
    c_r = rng.normal(size=20) + 1j * rng.normal(size=20)
    tdat_s = rng.normal(size=n) + 1j * rng.normal(size=n)
    t = lambda a: torch.from_numpy(np.asarray(a))
    return dict(nu=nu, x=[t(v) for v in x], grid=t(grid), data=t(data), src=[t(v) for v in src],
                tgt=[t(v) for v in tgt], c=t(c), tdat=t(tdat), tgt_s=[t(v) for v in tgt_s],
                src_r=[t(v) for v in src_r], c_r=t(c_r), tdat_s=t(tdat_s))


def _leaf(v):
    return v.clone().requires_grad_(True)


def _cases(rank, ws, ndim):
    """(name, single-process value and grads, this rank's sharded value and
    grads) for every pattern; sharded grads of sharded inputs are this
    rank's slice."""
    sys.path.insert(0, os.path.join(REPO, "jax-finufft_gb300"))
    from jax_finufft_gb300 import sharding as sh

    I = _inputs(ndim, ws)
    n = I["c"].shape[0]
    sl = slice(rank * n // ws, (rank + 1) * n // ws)
    out = []

    # type 2: grid replicated, points + data sharded; d/d grid and d/d x
    def loss2(g, pts, d, tf):
        return torch.sum(torch.abs(tf(g, *pts) - d) ** 2)

    g0, x0 = _leaf(I["grid"]), [_leaf(v) for v in I["x"]]
    L = loss2(g0, x0, I["data"], direct2)
    gr = torch.autograd.grad(L, [g0] + x0)
    g1, x1 = _leaf(I["grid"]), [_leaf(v[sl]) for v in I["x"]]
    Ll = loss2(g1, x1, I["data"][sl], lambda g, *p: sh.nufft2(g, *p, transform=direct2))
    gl = torch.autograd.grad(Ll, [g1] + x1)
    Ls = sh.reduce_sum(Ll.detach())
    out.append(("type2", [L, gr[0]] + [v[sl] for v in gr[1:]], [Ls] + list(gl)))

    # type 1: strengths + points sharded, outputs summed; d/d c and d/d x
    target = I["grid"]

    def loss1(f):
        return torch.sum(torch.abs(f - target) ** 2)

    c0, x0 = _leaf(I["c"]), [_leaf(v) for v in I["x"]]
    L = loss1(direct1(I["nu"], c0, *x0))
    gr = torch.autograd.grad(L, [c0] + x0)
    c1, x1 = _leaf(I["c"][sl]), [_leaf(v[sl]) for v in I["x"]]
    Ll = loss1(sh.nufft1(I["nu"], c1, *x1, transform=direct1))
    gl = torch.autograd.grad(Ll, [c1] + x1)
    out.append(("type1", [L] + [v[sl] for v in gr], [Ll] + list(gl)))

    # type 3, sources sharded, targets replicated; d/d c and d/d targets
    def loss3(f, d):
        return torch.sum(torch.abs(f - d) ** 2)

    c0, s0 = _leaf(I["c"]), [_leaf(v) for v in I["tgt"]]
    L = loss3(direct3(c0, *I["src"], *s0), I["tdat"])
    gr = torch.autograd.grad(L, [c0] + s0)
    c1, s1 = _leaf(I["c"][sl]), [_leaf(v) for v in I["tgt"]]
    Ll = loss3(sh.nufft3(c1, *[v[sl] for v in I["src"]], *s1, shard="sources",
                         transform=direct3), I["tdat"])
    gl = torch.autograd.grad(Ll, [c1] + s1)
    out.append(("type3_sources", [L, gr[0][sl]] + list(gr[1:]), [Ll] + list(gl)))

    # type 3, targets sharded, sources + strengths replicated; d/d c and d/d x
    c0, x0 = _leaf(I["c_r"]), [_leaf(v) for v in I["src_r"]]
    L = loss3(direct3(c0, *x0, *I["tgt_s"]), I["tdat_s"])
    gr = torch.autograd.grad(L, [c0] + x0)
    c1, x1 = _leaf(I["c_r"]), [_leaf(v) for v in I["src_r"]]
    Ll = loss3(sh.nufft3(c1, *x1, *[v[sl] for v in I["tgt_s"]], shard="targets",
                         transform=direct3), I["tdat_s"][sl])
    gl = torch.autograd.grad(Ll, [c1] + x1)
    Ls = sh.reduce_sum(Ll.detach())
    out.append(("type3_targets", [L] + list(gr), [Ls] + list(gl)))

    # forward values with the oracle port as the per-rank transform
    f_single = oracle_transform(1)(I["nu"], I["c"], *I["x"])
    f_shard = sh.nufft1(I["nu"], I["c"][sl], *[v[sl] for v in I["x"]],
                        transform=oracle_transform(1))
    out.append(("oracle_type1", [f_single], [f_shard]))
    v_single = oracle_transform(2)(I["grid"], *I["x"])[sl]
    v_shard = sh.nufft2(I["grid"], *[v[sl] for v in I["x"]], transform=oracle_transform(2))
    out.append(("oracle_type2", [v_single], [v_shard]))
    f_single = oracle_transform(3)(I["c"], *I["src"], *I["tgt"])
    f_shard = sh.nufft3(I["c"][sl], *[v[sl] for v in I["src"]], *I["tgt"], shard="sources",
                        transform=oracle_transform(3))
    out.append(("oracle_type3", [f_single], [f_shard]))
    with pytest.raises(NotImplementedError):
        sh.nufft3(I["c"][sl], *I["src"], *I["tgt"], shard="both", transform=direct3)
    return [(name, [a.detach().numpy() for a in s], [b.detach().numpy() for b in p])
            for name, s, p in out]


def _worker(rank, ws, port, ndim, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        q.put((rank, _cases(rank, ws, ndim)))
        dist.barrier()
    except Exception as e:  # report instead of hanging the other rank's queue read
        q.put((rank, repr(e)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_sharded_patterns_match_single_process(ndim):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, WS, port, ndim, q)) for r in range(WS)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in range(WS))
    for p in procs:
        p.join(timeout=60)
    for r in range(WS):
        assert not isinstance(res[r], str), res[r]
        assert procs[r].exitcode == 0
        for name, single, sharded in res[r]:
            assert len(single) == len(sharded), name
            for a, b in zip(sharded, single):
                np.testing.assert_allclose(a, b, rtol=1e-7, atol=1e-12 * max(1.0, np.abs(b).max()),
                                           err_msg="%s rank %d" % (name, r))


def test_single_rank_patterns_are_the_plain_transforms():
    """Without an initialised process group (one process), the collectives
    are not reached only when no gradient flows; check the shapes of the
    type-2 and type-3 (targets) forwards, which need no collective."""
    sys.path.insert(0, os.path.join(REPO, "jax-finufft_gb300"))
    from jax_finufft_gb300 import sharding as sh

    I = _inputs(2, 1)
    v = sh.nufft2(I["grid"], *I["x"], transform=direct2)
    np.testing.assert_allclose(v.numpy(), direct2(I["grid"], *I["x"]).numpy())
    f = sh.nufft3(I["c_r"], *I["src_r"], *I["tgt_s"], shard="targets", transform=direct3)
    assert f.shape == (I["tgt_s"][0].shape[0],)
    with pytest.raises(ValueError):
        sh.nufft3(I["c_r"], *I["src_r"], shard="nowhere", transform=direct3)
