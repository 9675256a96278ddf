"""GPU parity: the CUDA path against the golden known answers and the oracle.

Every call goes through libgbnufft.so's C ABI (gbn_run via the torch binding,
or the plan API through ctypes for the bit-exact fold/bin checks).
Tolerances:
  * golden cases: the reference tests' own comparison (tests/ops_test.py:14-16,
    120: elementwise rtol, jax's default atol, no floor), helpers.check_reference;
  * against the CPU oracle (same algorithm in FP64): relative l2 within
    5*max(eps, 1e-6) for FP32 compute and 5*eps for FP64 compute;
  * fold, grid starts, offsets and bin indices: bit-exact.
"""
import ctypes
from itertools import product

import numpy as np
import pytest
import torch

from helpers import ORACLE_HELD, check_close, check_reference, golden, rel_l2

pytestmark = pytest.mark.gpu

DEV = "cuda"


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


@pytest.fixture(scope="module")
def jf(native):
    import jax_finufft_gb300

    return jax_finufft_gb300


@pytest.fixture(scope="module")
def cn(oracle_lib):
    from oracle import cpu_nufft

    return cpu_nufft


FWD = list(product([1, 2, 3], [False, True], [-1, 1]))


def _key(ndim, x64, iflag):
    return "d%d_%s_i%+d" % (ndim, "x64" if x64 else "x32", iflag)


# --------------------------------------------------------------------------
# known answers of the reference's tests
# --------------------------------------------------------------------------
@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_nufft1_forward(jf, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t1_" + _key(ndim, x64, iflag)
    x, c, f = g[k + "_x"], g[k + "_c"], g[k + "_f"]
    eps = 1e-10 if x64 else 1e-7
    out = jf.nufft1(f.shape, T(c), *[T(v) for v in x], eps=eps, iflag=iflag)
    assert out.dtype == (torch.complex128 if x64 else torch.complex64)
    held = None
    if (1, ndim, x64, iflag) in ORACLE_HELD:
        from oracle import cpu_nufft

        held = cpu_nufft.nufft1(f.shape, c, *x, eps=eps, iflag=iflag)
    check_reference(out.cpu().numpy(), f, held=held)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_nufft2_forward(jf, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t2_" + _key(ndim, x64, iflag)
    x, f, c = g[k + "_x"], g[k + "_f"], g[k + "_c"]
    eps = 1e-10 if x64 else 1e-7
    out = jf.nufft2(T(f), *[T(v) for v in x], eps=eps, iflag=iflag)
    check_reference(out.cpu().numpy(), c)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_nufft3_forward(jf, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t3_" + _key(ndim, x64, iflag)
    x, s, c, f = g[k + "_x"], g[k + "_s"], g[k + "_c"], g[k + "_f"]
    eps = 1e-10 if x64 else 1e-7
    out = jf.nufft3(T(c), *[T(v) for v in x], *[T(v) for v in s], eps=eps, iflag=iflag)
    check_reference(out.cpu().numpy(), f,
                    rtol=float(g["t3_rtol_complex128"] if x64 else g["t3_rtol_complex64"]))


@pytest.mark.parametrize("mo, nf, ndim, ty", list(product([0, 1], [16, 17], [1, 2, 3], [1, 2])))
def test_modeord(jf, mo, nf, ndim, ty):
    from jax_finufft_gb300.options import Opts

    g = golden("modeord.npz")
    k = "mo%d_n%d_d%d_t%d" % (mo, nf, ndim, ty)
    x = g[k + "_x"]
    opts = Opts(modeord=mo)
    if ty == 1:
        c, f = g[k + "_c"], g[k + "_f"]
        out = jf.nufft1(f.shape, T(c), *[T(v) for v in x], eps=1e-10, iflag=1, opts=opts)
        check_reference(out.cpu().numpy(), f)
    else:
        f, c = g[k + "_f"], g[k + "_c"]
        out = jf.nufft2(T(f), *[T(v) for v in x], eps=1e-10, iflag=1, opts=opts)
        check_reference(out.cpu().numpy(), c)


def test_multi_transform(jf):
    """(n_tot, n_tr, ...) inputs: n_tot setpts/execute rounds in one call."""
    g = golden("multi.npz")
    n_k = int(g["n_k"])
    x = T(g["x"])
    out1 = jf.nufft1(n_k, T(g["c"]), x)
    out2 = jf.nufft2(T(g["f"]), x)
    out3 = jf.nufft3(T(g["c"]), x, T(g["xt"]))
    check_reference(out1.cpu().numpy(), g["t1"], rtol=1e-4)
    check_reference(out2.cpu().numpy(), g["t2"], rtol=1e-4)
    check_reference(out3.cpu().numpy(), g["t3"], rtol=1e-4)
    for n in range(g["c"].shape[1]):
        check_close(out1[:, n].cpu().numpy(), jf.nufft1(n_k, T(g["c"][:, n]), x).cpu().numpy(),
                    rtol=1e-4)


# --------------------------------------------------------------------------
# against the CPU oracle: every dimension, type, precision and method
# --------------------------------------------------------------------------
SHAPES = {1: (97,), 2: (40, 33), 3: (20, 17, 24)}


def _points(rng, ndim, M, kind):
    if kind == "uniform":
        return [rng.uniform(-np.pi, np.pi, M) for _ in range(ndim)]
    if kind == "cluster":
        return [rng.normal(0.0, 0.1, M) for _ in range(ndim)]
    return [rng.normal(0.0, 1.0, M) * 7.0 for _ in range(ndim)]  # far outside one period


def _tol(eps, single):
    return 5 * max(eps, 1e-6) if single else 5 * eps


def _opts(**kw):
    from jax_finufft_gb300.options import Opts

    return Opts(**kw)


CASES = []
for _ndim, _ty, _single in product([1, 2, 3], [1, 2, 3], [True, False]):
    CASES.append((_ndim, _ty, _single, {}, "uniform"))
for _ndim, _ty in product([2, 3], [1, 2]):
    CASES += [
        (_ndim, _ty, True, dict(gpu_method=1), "uniform"),
        (_ndim, _ty, True, dict(gpu_method=1, gpu_sort=False), "uniform"),
        (_ndim, _ty, True, dict(gpu_kerevalmeth=False), "uniform"),
        (_ndim, _ty, True, dict(gpu_maxsubprobsize=32), "cluster"),
        (_ndim, _ty, False, dict(gpu_upsampfac=1.25), "wide"),
        (_ndim, _ty, False, dict(modeord=1, gpu_method=2), "wide"),
        (_ndim, _ty, True, dict(gpu_binsizex=8, gpu_binsizey=8, gpu_binsizez=4), "cluster"),
    ]
# narrow kernels (w = 3, 4): six-lane groups with idle lanes inside the group
for _ndim, _ty in product([1, 2, 3], [1, 2]):
    CASES.append((_ndim, _ty, True, dict(_eps=1e-2 if _ty == 1 else 1e-3), "cluster"))
CASES += [(1, 1, True, dict(gpu_upsampfac=1.25), "cluster"),
          (1, 2, False, dict(gpu_method=1), "wide"),
          (3, 1, False, dict(gpu_method=2), "uniform"),
          (3, 2, False, dict(gpu_method=1), "uniform"),
          (2, 1, False, dict(gpu_precision=1), "uniform"),
          (2, 2, False, dict(gpu_precision=3), "uniform")]
# Kaiser-Bessel kernel shape: every dimension and type in both precisions,
# and its direct evaluation (I0 on the device) in place of the polynomials
for _ndim, _ty, _single in product([1, 2, 3], [1, 2, 3], [True, False]):
    CASES.append((_ndim, _ty, _single, dict(gpu_kernel=1), "uniform"))
CASES += [(2, 1, True, dict(gpu_kernel=1, gpu_kerevalmeth=False), "cluster"),
          (3, 2, False, dict(gpu_kernel=1, gpu_kerevalmeth=False), "uniform")]


@pytest.mark.parametrize("ndim, ty, single, kw, kind", CASES,
                         ids=["d%d-t%d-%s-%s-%s" % (c[0], c[1], "f" if c[2] else "d",
                                                    "_".join("%s=%s" % i for i in c[3].items()) or "default",
                                                    c[4]) for c in CASES])
def test_against_oracle(jf, cn, ndim, ty, single, kw, kind):
    rng = np.random.default_rng(100 * ndim + 10 * ty + int(single))
    M = 3000
    eps = 1e-5 if single else 1e-9
    if kw.get("gpu_precision") == 3:
        eps = 1e-6
    kw = dict(kw)
    eps = kw.pop("_eps", eps)
    rdt, cdt = (np.float32, np.complex64) if single else (np.float64, np.complex128)
    opts = _opts(**kw)
    mo = int(kw.get("modeord", 0))
    sigma = kw.get("gpu_upsampfac", 2.0)
    kern = int(kw.get("gpu_kernel", 0))
    x = [v.astype(rdt) for v in _points(rng, ndim, M, kind)]
    iflag = 1 if (ndim + ty) % 2 else -1
    if ty == 1:
        c = (rng.normal(size=(2, M)) + 1j * rng.normal(size=(2, M))).astype(cdt)
        out = jf.nufft1(SHAPES[ndim], T(c), *[T(v) for v in x], eps=eps, iflag=iflag, opts=opts)
        ref = cn.nufft1(SHAPES[ndim], c, *x, eps=eps, iflag=iflag, modeord=mo, sigma=sigma,
                        kernel=kern)
    elif ty == 2:
        f = (rng.normal(size=(2,) + SHAPES[ndim]) + 1j * rng.normal(size=(2,) + SHAPES[ndim])
             ).astype(cdt)
        out = jf.nufft2(T(f), *[T(v) for v in x], eps=eps, iflag=iflag, opts=opts)
        ref = cn.nufft2(f, *x, eps=eps, iflag=iflag, modeord=mo, sigma=sigma, kernel=kern)
    else:
        s = [rng.uniform(-20, 20, 700).astype(rdt) for _ in range(ndim)]
        c = (rng.normal(size=(2, M)) + 1j * rng.normal(size=(2, M))).astype(cdt)
        out = jf.nufft3(T(c), *[T(v) for v in x], *[T(v) for v in s], eps=eps, iflag=iflag,
                        opts=opts)
        ref = cn.nufft3(c, *x, *s, eps=eps, iflag=iflag, sigma=sigma, kernel=kern)
    out = out.cpu().numpy()
    assert out.shape == ref.shape
    assert np.isfinite(out).all()
    comp_single = single or kw.get("gpu_precision") in (1, 3)
    assert rel_l2(out, ref) < _tol(eps, comp_single), rel_l2(out, ref)


# --------------------------------------------------------------------------
# bit-exact fold, grid starts, offsets and bins (plan API through ctypes)
# --------------------------------------------------------------------------
def _plan(native, ty, ndim, nmodes, single, opts, stream=None):
    from jax_finufft_gb300 import _native

    plan = ctypes.c_void_p()
    nm = (ctypes.c_int64 * 3)(*(list(nmodes) + [1] * (3 - len(nmodes))))
    mk = native.gbnf_makeplan if single else native.gbn_makeplan
    rc = mk(ty, ndim, nm, 1, 1, 1e-6, ctypes.byref(plan), ctypes.byref(opts), stream)
    _native.check(rc)
    return plan


def _boundary_points(rng, nf, M, rdt):
    """Coordinates on and next to fine-grid cells and half cells (where the
    fold's ceiling and the FP32 rounding of the offset are closest to a
    decision), their float neighbours, and special values (+-pi, 0, tiny,
    large) -- the points the FP32 fold's integer fast path hands to the FP64
    chain, mixed into warps with points it keeps."""
    out = []
    for n in nf:
        j = rng.integers(-n, n, M).astype(np.float64)
        off = rng.choice([0.0, 0.5], M)
        tiny = (rng.random(M) - 0.5) * np.ldexp(1.0, -rng.integers(0, 45, M))
        v = (2 * np.pi * (j + off + tiny) / n).astype(rdt)
        k = M // 8
        steps = rng.integers(-40, 41, k)
        v[k:2 * k] = v[k:2 * k] + steps * np.spacing(v[k:2 * k])
        v[:k] = rng.choice(np.array([np.pi, -np.pi, 0.0, 1e-30, -1e-30, 2 * np.pi, 1e4, -3e5]), k)
        out.append(v.astype(rdt))
    return out


@pytest.mark.parametrize("ndim, single, kind", list(product([1, 2, 3], [True, False],
                                                            ["uniform", "cluster", "wide",
                                                             "boundary"])))
def test_fold_and_bins_bit_exact(native, cn, ndim, single, kind):
    from jax_finufft_gb300 import _native

    rng = np.random.default_rng(7 + ndim)
    M = 20000
    rdt = np.float32 if single else np.float64
    nmodes = {1: (1000,), 2: (200, 130), 3: (40, 50, 36)}[ndim]
    opts = _native.default_opts()
    bs = {1: (128, 1, 1), 2: (16, 32, 1), 3: (8, 16, 4)}[ndim]
    opts.gpu_binsizex, opts.gpu_binsizey, opts.gpu_binsizez = bs
    opts.gpu_method = 2
    plan = _plan(native, 1, ndim, nmodes, single, opts)
    try:
        w = ctypes.c_int()
        nf = (ctypes.c_int64 * 3)()
        _native.check(native.gbn_plan_info(plan, ctypes.byref(w), nf, None, None))
        if kind == "boundary":
            x = _boundary_points(rng, [nf[d] for d in range(ndim)], M, rdt)
        else:
            x = [v.astype(rdt) for v in _points(rng, ndim, M, kind)]
            x[0][:4] = np.array([np.pi, -np.pi, 0.0, 2 * np.pi], dtype=rdt)
        xt = [T(v) for v in x] + [None] * (3 - ndim)
        ptr = [ctypes.c_void_p(t.data_ptr()) if t is not None else None for t in xt]
        setpts = native.gbnf_setpts if single else native.gbn_setpts
        torch.cuda.synchronize()
        _native.check(setpts(plan, M, ptr[0], ptr[1], ptr[2], 0, None, None, None))
        nbins = ctypes.c_int64()
        native.gbn_debug_bins(plan, None, None, ctypes.byref(nbins))
        bins = np.empty(M, dtype=np.int64)
        counts = np.empty(nbins.value, dtype=np.int64)
        _native.check(native.gbn_debug_bins(plan, bins.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                            counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                            ctypes.byref(nbins)))
        i0 = np.empty((M, 3), dtype=np.int64)
        de = np.empty((M, 3), dtype=np.float64)
        _native.check(native.gbn_debug_fold(plan, i0.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                            de.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    finally:
        native.gbn_destroy(plan)
    nf_b = [nf[d] for d in range(ndim)]
    bs_b = [min(bs[d], nf_b[d]) for d in range(ndim)]
    X, ri0, rde, rbin = cn.fold_points([v.astype(np.float64) for v in x], nf_b, w.value, bs_b)
    np.testing.assert_array_equal(bins, rbin)
    np.testing.assert_array_equal(i0[:, :ndim], ri0[:, :ndim])
    if single:
        np.testing.assert_array_equal(de[:, :ndim].astype(np.float32),
                                      rde[:, :ndim].astype(np.float32))
    else:
        np.testing.assert_array_equal(de[:, :ndim], rde[:, :ndim])
    np.testing.assert_array_equal(counts, np.bincount(rbin, minlength=nbins.value))


@pytest.mark.parametrize("ndim", [2, 3])
def test_spread_dynamic_range(jf, cn, ndim):
    """FP32 shared-memory spreading accumulates in 32-bit fixed point scaled
    per subproblem: strengths spanning 8 orders of magnitude in separate
    regions must each keep FP32-level accuracy (checked per region by a
    type-1 transform of each region alone against the oracle)."""
    rng = np.random.default_rng(5)
    M = 4000
    shape = SHAPES[ndim]
    x_big = [rng.normal(-1.5, 0.2, M).astype(np.float32) for _ in range(ndim)]
    x_small = [rng.normal(1.5, 0.2, M).astype(np.float32) for _ in range(ndim)]
    c_big = (1e4 * (rng.normal(size=M) + 1j * rng.normal(size=M))).astype(np.complex64)
    c_small = (1e-4 * (rng.normal(size=M) + 1j * rng.normal(size=M))).astype(np.complex64)
    x = [np.concatenate([a, b]) for a, b in zip(x_big, x_small)]
    c = np.concatenate([c_big, c_small])
    eps = 1e-6
    both = jf.nufft1(shape, T(c), *[T(v) for v in x], eps=eps).cpu().numpy()
    small_only = jf.nufft1(shape, T(np.concatenate([0 * c_big, c_small])), *[T(v) for v in x],
                           eps=eps).cpu().numpy()
    ref_small = cn.nufft1(shape, c_small, *x_small, eps=eps)
    ref_both = cn.nufft1(shape, c, *x, eps=eps)
    assert rel_l2(both, ref_both) < 5e-6
    assert rel_l2(small_only, ref_small) < 5e-6
