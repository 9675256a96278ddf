"""The row-owned FP32 spreads at every width they serve, against the oracle.

spread_rows_kernel serves 3D FP32 type-1 plans with bins 16 x 16 x bz and
kernel widths 4..8 (one template instance per width); spread_rows2_kernel
2D plans of four or more stacked transforms with bins 16 x 16 (the type-1
FP32 default) or 32 x 32, four transforms per block.  Both round each contribution to the
fixed-point tile by one FFMA where the tolerance is >= 1e-5 or a
subproblem's strengths sum to >= 512 times the largest; otherwise the 3D
kernel uses the FP32-to-int32 conversion and the 2D kernel integer products
(int32 strengths times Q30 kernel products).  Each case runs a type-1 transform through the
library on complex64 data and compares it with the FP64 oracle
(oracle/cpu_nufft.py) in relative l2 within 5 max(eps, 1e-6), the bound of
the other GPU parity tests.  Points: half uniform, half in a tight cluster,
so that tiles inside the grid (bulk reduce-add), tiles that wrap (per-cell
atomics), sparse and dense subproblems all occur.
"""
import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu

SHAPE = (40, 36, 44)  # fine grid 80 x 72 x 88: bins 16 x 16 x 12 cover it with interior and wrapping tiles
SHAPE2 = (60, 52)  # fine grid 120 x 104: bins 32 x 32 (or 16 x 32) give interior and wrapping tiles


def _inputs(seed, M, unit_strengths=False, dim=3, T=None):
    rng = np.random.default_rng(seed)
    h = M // 2
    x = [np.concatenate([rng.uniform(-np.pi, np.pi, h), rng.normal(0.3, 0.05, M - h)])
         for _ in range(dim)]
    shape = (M,) if T is None else (T, M)
    if unit_strengths:
        c = np.exp(2j * np.pi * rng.uniform(size=shape))
    else:
        c = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    return x, c


@pytest.mark.parametrize("eps", [1e-3, 1e-4, 1e-5, 1e-6, 1e-7])
@pytest.mark.parametrize("kernel", [0, 1])
def test_row_spread_widths_match_oracle(eps, kernel):
    import jax_finufft_gb300 as jf
    from jax_finufft_gb300.options import Opts
    from oracle import cpu_nufft as cn

    x, c = _inputs(17, 40000)
    out = jf.nufft1(SHAPE, torch.tensor(c.astype(np.complex64), device="cuda"),
                    *[torch.tensor(v.astype(np.float32), device="cuda") for v in x],
                    eps=eps, iflag=1, opts=Opts(gpu_kernel=kernel)).cpu().numpy()
    ref = cn.nufft1(SHAPE, c, *[v.astype(np.float32).astype(np.float64) for v in x], eps=eps,
                    iflag=1, kernel=kernel)
    assert np.isfinite(out).all()
    assert rel_l2(out, ref) < 5 * max(eps, 1e-6), rel_l2(out, ref)


def test_row_spread_dense_unit_strengths():
    """eps 1e-6 (conversion rounding by default) with unit-modulus strengths
    in a dense cluster: full subproblems sum to 1024 times their largest
    strength, so they take the FFMA rounding; sparse ones the conversion."""
    import jax_finufft_gb300 as jf
    from oracle import cpu_nufft as cn

    x, c = _inputs(29, 60000, unit_strengths=True)
    eps = 1e-6
    out = jf.nufft1(SHAPE, torch.tensor(c.astype(np.complex64), device="cuda"),
                    *[torch.tensor(v.astype(np.float32), device="cuda") for v in x],
                    eps=eps, iflag=-1).cpu().numpy()
    ref = cn.nufft1(SHAPE, c, *[v.astype(np.float32).astype(np.float64) for v in x], eps=eps,
                    iflag=-1)
    assert rel_l2(out, ref) < 5 * max(eps, 1e-6), rel_l2(out, ref)


@pytest.mark.parametrize("eps", [1e-3, 1e-4, 1e-5, 1e-6, 1e-7])
@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("T", [None, 6])
def test_row_spread_2d_widths_match_oracle(eps, kernel, T):
    """2D: one transform (the G-lane kernel, which serves fewer than four
    stacked transforms) and six stacked transforms (row-owned blocks of four,
    then a block of two)."""
    import jax_finufft_gb300 as jf
    from jax_finufft_gb300.options import Opts
    from oracle import cpu_nufft as cn

    x, c = _inputs(23, 30000, dim=2, T=T)
    out = jf.nufft1(SHAPE2, torch.tensor(c.astype(np.complex64), device="cuda"),
                    *[torch.tensor(v.astype(np.float32), device="cuda") for v in x],
                    eps=eps, iflag=1, opts=Opts(gpu_kernel=kernel)).cpu().numpy()
    ref = cn.nufft1(SHAPE2, c, *[v.astype(np.float32).astype(np.float64) for v in x], eps=eps,
                    iflag=1, kernel=kernel)
    assert np.isfinite(out).all()
    assert rel_l2(out, ref) < 5 * max(eps, 1e-6), rel_l2(out, ref)


@pytest.mark.parametrize("bins,maxsub", [((32, 32), 0), ((32, 32), 40), ((16, 32), 0)])
def test_row_spread_2d_bins_and_small_subproblems(bins, maxsub):
    """Bins 32 x 32 (the wider row layout; type-1 FP32 plans default to
    16 x 16); subproblems too small for the row-owned kernel's zero-add reach
    (maxsub 40 < 2 * 40 + 2 cells); bins 16 x 32, which it does not serve:
    the last two take the G-lane kernel.  All against the oracle."""
    import jax_finufft_gb300 as jf
    from jax_finufft_gb300.options import Opts
    from oracle import cpu_nufft as cn

    x, c = _inputs(31, 20000, dim=2, T=4)
    eps = 1e-6
    opts = Opts(gpu_binsizex=bins[0], gpu_binsizey=bins[1], gpu_maxsubprobsize=maxsub)
    out = jf.nufft1(SHAPE2, torch.tensor(c.astype(np.complex64), device="cuda"),
                    *[torch.tensor(v.astype(np.float32), device="cuda") for v in x],
                    eps=eps, iflag=-1, opts=opts).cpu().numpy()
    ref = cn.nufft1(SHAPE2, c, *[v.astype(np.float32).astype(np.float64) for v in x], eps=eps,
                    iflag=-1)
    assert rel_l2(out, ref) < 5 * max(eps, 1e-6), rel_l2(out, ref)


def test_row_spread_2d_dense_unit_strengths():
    """Four stacked transforms of unit-modulus strengths in a dense cluster at
    eps 1e-6: full subproblems (integer strengths near 2^33 / 1024, the sum
    bound) beside sparse ones (near 2^31, the maximum bound)."""
    import jax_finufft_gb300 as jf
    from oracle import cpu_nufft as cn

    x, c = _inputs(37, 60000, unit_strengths=True, dim=2, T=4)
    eps = 1e-6
    out = jf.nufft1(SHAPE2, torch.tensor(c.astype(np.complex64), device="cuda"),
                    *[torch.tensor(v.astype(np.float32), device="cuda") for v in x],
                    eps=eps, iflag=1).cpu().numpy()
    ref = cn.nufft1(SHAPE2, c, *[v.astype(np.float32).astype(np.float64) for v in x], eps=eps,
                    iflag=1)
    assert rel_l2(out, ref) < 5 * max(eps, 1e-6), rel_l2(out, ref)
