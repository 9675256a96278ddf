"""Repeated per-call transforms replayed from CUDA graphs (gbn_run).

The per-call driver keeps its plans; a call whose arguments (sizes and
buffers) repeat those of a recent call is captured once into a CUDA graph
and later identical calls replay it.  The replays read the buffers' current
contents: with the strengths, modes or points changed in place between
calls, every call must still match the FP64 oracle (oracle/cpu_nufft.py) on
the current contents, in relative l2 within 5 max(eps, 1e-6), the bound of
the other GPU parity tests.  Alternating output buffers, a call of other
sizes in between (which drops the graphs) and a call inside the caller's own
stream capture (which joins that capture) are covered too.
"""
import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_type1_replays_follow_in_place_updates(dtype):
    import jax_finufft_gb300 as jf
    from oracle import cpu_nufft as cn

    rdt = torch.float32 if dtype == torch.complex64 else torch.float64
    g = torch.Generator(device="cuda").manual_seed(3)
    M, shape, eps = 5000, (40, 36), 1e-6
    x = [(torch.rand(M, generator=g, device="cuda", dtype=rdt) * 2 - 1) * np.pi for _ in range(2)]
    c = torch.randn(M, generator=g, device="cuda", dtype=dtype)
    for step in range(6):
        out = jf.nufft1(shape, c, *x, eps=eps)  # from the third call on: replays
        torch.cuda.synchronize()
        ref = cn.nufft1(shape, _np(c).astype(np.complex128),
                        *[_np(v).astype(np.float64) for v in x], eps=eps, iflag=1)
        assert rel_l2(_np(out), ref) < 5 * max(eps, 1e-6), (step, rel_l2(_np(out), ref))
        c.mul_(1.5).add_(0.25j)  # new contents, same buffers
        x[step % 2].mul_(0.9)


def test_type2_replays_with_alternating_outputs_and_other_sizes():
    import jax_finufft_gb300 as jf
    from oracle import cpu_nufft as cn

    g = torch.Generator(device="cuda").manual_seed(5)
    eps = 1e-5
    f = torch.randn(32, 24, 20, generator=g, device="cuda", dtype=torch.complex64)
    xs = {M: [(torch.rand(M, generator=g, device="cuda") * 2 - 1) * np.pi for _ in range(3)]
          for M in (3000, 4500)}
    kept = []
    for step in range(8):
        M = 3000 if step != 5 else 4500  # one call of another size in between
        out = jf.nufft2(f, *xs[M], eps=eps)
        kept.append(out)  # outputs kept alive: the output buffers alternate
        torch.cuda.synchronize()
        ref = cn.nufft2(_np(f).astype(np.complex128), *[_np(v).astype(np.float64) for v in xs[M]],
                        eps=eps, iflag=-1)
        assert rel_l2(_np(out), ref) < 5 * eps, (step, rel_l2(_np(out), ref))
        f.mul_(-1.0).add_(0.5)
        if len(kept) > 2:
            kept.pop(0)


def test_call_inside_a_caller_capture_joins_it():
    import jax_finufft_gb300 as jf
    from oracle import cpu_nufft as cn

    g = torch.Generator(device="cuda").manual_seed(7)
    M, shape, eps = 4000, (24, 20, 16), 1e-5
    x = [(torch.rand(M, generator=g, device="cuda") * 2 - 1) * np.pi for _ in range(3)]
    c = torch.randn(M, generator=g, device="cuda", dtype=torch.complex64)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):  # the library's own graph for these arguments exists
            jf.nufft1(shape, c, *x, eps=eps)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):  # the stream the plan was made for
        out = jf.nufft1(shape, c, *x, eps=eps)
    c.mul_(2.0)
    graph.replay()
    torch.cuda.synchronize()
    ref = cn.nufft1(shape, _np(c).astype(np.complex128), *[_np(v).astype(np.float64) for v in x],
                    eps=eps, iflag=1)
    assert rel_l2(_np(out), ref) < 5 * eps, rel_l2(_np(out), ref)
