"""The CPU oracle pinned against the reference tests' known answers.

The reference's tests (tests/ops_test.py) check every transform against a
direct NUDFT sum computed in the test; tests/golden holds those sums as the
reference's own test code computed them (tests/golden/from_reference.py runs
that code with jax stubbed out).  The oracle -- the FP64 direct sums of
oracle/direct.py and the CPU restatement of the fast algorithm -- must
reproduce them, the fast algorithm at the reference's own tolerances with
its elementwise comparison (no absolute floor), before it is trusted as the
checker for the GPU path.
"""
from itertools import product

import numpy as np
import pytest

from helpers import ORACLE_HELD, ATOL, RTOL, check_reference, golden, rel_l2


@pytest.fixture(scope="module")
def cn(oracle_lib):
    from oracle import cpu_nufft

    return cpu_nufft


FWD = list(product([1, 2, 3], [False, True], [-1, 1]))


def _key(ndim, x64, iflag):
    return "d%d_%s_i%+d" % (ndim, "x64" if x64 else "x32", iflag)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_oracle_nufft1_golden(cn, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t1_" + _key(ndim, x64, iflag)
    x, c, f = g[k + "_x"], g[k + "_c"], g[k + "_f"]
    eps = 1e-10 if x64 else 1e-7
    out = cn.nufft1(f.shape, c.astype(np.complex128), *x.astype(np.float64), eps=eps, iflag=iflag)
    if (1, ndim, x64, iflag) in ORACLE_HELD:
        # the documented miss: one entry of 26,250, by less than 3x its bound
        ratio = np.abs(out - f) / (ATOL["complex128"] + RTOL["complex128"] * np.abs(f))
        assert np.sum(ratio > 1) == 1 and ratio.max() < 3.0, (np.sum(ratio > 1), ratio.max())
        assert rel_l2(out, f) <= RTOL["complex128"]
        return
    check_reference(out.astype(c.dtype), f)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_oracle_nufft2_golden(cn, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t2_" + _key(ndim, x64, iflag)
    x, f, c = g[k + "_x"], g[k + "_f"], g[k + "_c"]
    eps = 1e-10 if x64 else 1e-7
    out = cn.nufft2(f.astype(np.complex128), *x.astype(np.float64), eps=eps, iflag=iflag)
    check_reference(out.astype(f.dtype), c)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_oracle_nufft3_golden(cn, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t3_" + _key(ndim, x64, iflag)
    x, s, c, f = g[k + "_x"], g[k + "_s"], g[k + "_c"], g[k + "_f"]
    eps = 1e-10 if x64 else 1e-7
    out = cn.nufft3(c.astype(np.complex128), *x.astype(np.float64), *s.astype(np.float64),
                    eps=eps, iflag=iflag)
    check_reference(out.astype(c.dtype), f,
                    rtol=float(g["t3_rtol_complex128"] if x64 else g["t3_rtol_complex64"]))


@pytest.mark.parametrize("mo, nf, ndim, ty", list(product([0, 1], [16, 17], [1, 2, 3], [1, 2])))
def test_oracle_modeord_golden(cn, mo, nf, ndim, ty):
    g = golden("modeord.npz")
    k = "mo%d_n%d_d%d_t%d" % (mo, nf, ndim, ty)
    x = g[k + "_x"]
    if ty == 1:
        c, f = g[k + "_c"], g[k + "_f"]
        out = cn.nufft1(f.shape, c, *x, eps=1e-10, iflag=1, modeord=mo)
        check_reference(out, f)
    else:
        f, c = g[k + "_f"], g[k + "_c"]
        out = cn.nufft2(f, *x, eps=1e-10, iflag=1, modeord=mo)
        check_reference(out, c)


def test_oracle_multi_golden(cn):
    g = golden("multi.npz")
    n_k = int(g["n_k"])
    for i in range(g["x"].shape[0]):
        check_reference(cn.nufft1((n_k,), g["c"][i], g["x"][i], eps=1e-6, iflag=1), g["t1"][i],
                        rtol=1e-4)
        check_reference(cn.nufft2(g["f"][i], g["x"][i], eps=1e-6, iflag=-1), g["t2"][i],
                        rtol=1e-4)
        check_reference(cn.nufft3(g["c"][i], g["x"][i], g["xt"][i], eps=1e-6, iflag=-1),
                        g["t3"][i], rtol=1e-4)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_direct_sums_match_reference_code(ndim, x64, iflag):
    """oracle/direct.py (the FP64 direct sums the GPU tests compare with at
    other sizes) reproduces the reference tests' own known answers: to
    round-off for float64; for float32 to the precision the reference's
    test computes in (its type-2 sum multiplies in place into a complex64
    array, ops_test.py:76-84, so its terms carry complex64 rounding)."""
    from oracle import direct

    g = golden("forward.npz")
    k = _key(ndim, x64, iflag)
    tol = 1e-13 if x64 else 1e-6
    x, c, f = g["t1_" + k + "_x"], g["t1_" + k + "_c"], g["t1_" + k + "_f"]
    got = [(direct.type1(c, list(x), f.shape, iflag), f)]
    x, f, c = g["t2_" + k + "_x"], g["t2_" + k + "_f"], g["t2_" + k + "_c"]
    got.append((direct.type2(f, list(x), iflag), c))
    x, s, c, f = (g["t3_" + k + "_x"], g["t3_" + k + "_s"], g["t3_" + k + "_c"],
                  g["t3_" + k + "_f"])
    got.append((direct.type3(c, list(x), list(s), iflag), f))
    for a, b in got:
        rms = float(np.sqrt(np.mean(np.abs(b) ** 2)))
        np.testing.assert_allclose(a.astype(b.dtype), b, rtol=tol, atol=tol * rms)


@pytest.mark.parametrize("mo, nf, ndim, ty", list(product([0, 1], [16, 17], [1, 2, 3], [1, 2])))
def test_direct_sums_match_reference_modeord(mo, nf, ndim, ty):
    from oracle import direct

    g = golden("modeord.npz")
    k = "mo%d_n%d_d%d_t%d" % (mo, nf, ndim, ty)
    x = g[k + "_x"]
    if ty == 1:
        a, b = direct.type1(g[k + "_c"], list(x), g[k + "_f"].shape, 1, modeord=mo), g[k + "_f"]
    else:
        a, b = direct.type2(g[k + "_f"], list(x), 1, modeord=mo), g[k + "_c"]
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-13 * float(np.abs(b).max()))


@pytest.mark.parametrize("eps", [1e-3, 1e-6, 1e-9, 1e-12])
@pytest.mark.parametrize("sigma", [2.0, 1.25])
def test_oracle_error_tracks_eps(cn, eps, sigma):
    """Relative l2 error vs the direct sum stays within a small multiple of eps."""
    from oracle import direct

    if cn.kernel_params(eps, sigma)[2]:
        pytest.skip("tolerance below what width 16 reaches at this sigma (warning case)")
    rng = np.random.default_rng(1)
    x = [rng.uniform(-np.pi, np.pi, 400) for _ in range(2)]
    c = rng.normal(size=400) + 1j * rng.normal(size=400)
    out = cn.nufft1((24, 31), c, *x, eps=eps, iflag=1, sigma=sigma)
    assert rel_l2(out, direct.type1(c, x, (24, 31), 1)) < 10 * eps


def test_oracle_points_outside_period(cn):
    """Points far outside [-pi, pi) fold periodically (ops_test.py:464 uses N(0,1))."""
    from oracle import direct

    rng = np.random.default_rng(2)
    x = rng.normal(size=300) * 50.0
    c = rng.normal(size=300) + 1j * rng.normal(size=300)
    out = cn.nufft1((40,), c, x, eps=1e-9, iflag=-1)
    assert rel_l2(out, direct.type1(c, [x], (40,), -1)) < 1e-8


def test_horner_fit_accuracy(cn):
    """The piecewise-polynomial fit (degree w+2) matches the kernel to ~e^-beta."""
    for sigma in (2.0, 1.25):
        for w in range(2, 17):
            if sigma == 2.0:
                beta = {2: 2.20, 3: 2.26, 4: 2.38}.get(w, 2.30) * w
            else:
                beta = 0.97 * np.pi * (1 - 1 / (2 * sigma)) * w
            coef = cn.horner_fit(w, beta, w + 2)
            d = np.linspace(0, 1, 257)[:-1]
            u = 2 * d - 1
            worst = 0.0
            for j in range(w):
                fit = np.polynomial.polynomial.polyval(u, coef[j])
                exact = cn.kernel(j - w / 2 + d, w, beta)
                worst = max(worst, np.max(np.abs(fit - exact)))
            assert worst < max(np.exp(-beta), 1e-14) * 2.0, (sigma, w, worst)


def test_kernel_params_rule(cn):
    assert cn.kernel_params(1e-6, 2.0)[0] == 7
    assert cn.kernel_params(1e-5, 2.0)[0] == 6
    assert cn.kernel_params(1e-12, 2.0)[0] == 13
    assert cn.kernel_params(1e-20, 2.0) [0] == 16 and cn.kernel_params(1e-20, 2.0)[2] == 1
    assert cn.fine_size(256, 2.0, 7) == 512
    assert cn.fine_size(75, 2.0, 8) == 150
    assert cn.next235even(1001) == 1024 and cn.next235even(7) == 8 and cn.next235even(2) == 2


def test_fold_edges(cn):
    nf = 512
    assert cn.lib().orc_fold(0.0, nf) == 0.0
    assert cn.lib().orc_fold(np.pi, nf) == 256.0
    assert 0.0 <= cn.lib().orc_fold(-np.pi, nf) < nf
    assert cn.lib().orc_fold(float("nan"), nf) == 0.0
    assert cn.lib().orc_fold(float("inf"), nf) == 0.0
    assert 0.0 <= cn.lib().orc_fold(1e300, nf) < nf
    assert 0.0 <= cn.lib().orc_fold(-1e-300, nf) < nf


@pytest.mark.parametrize("shape", [(40,), (33, 20), (20, 17, 24), (64, 64, 64)])
@pytest.mark.parametrize("mo", [0, 1])
def test_single_precision_path_matches_fp64(cn, shape, mo):
    """The timed CPU baseline (single-precision fast path: Horner kernel,
    coloured bin subgrids, complex64 FFT) against the FP64 oracle on the same
    points: agreement to single-precision round-off."""
    rng = np.random.default_rng(len(shape) + 10 * mo)
    M = 5000
    x = [np.concatenate([rng.uniform(-np.pi, np.pi, M // 2), rng.normal(0, 0.1, M - M // 2)])
         for _ in shape]
    c = rng.normal(size=M) + 1j * rng.normal(size=M)
    f = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    a = cn.nufft1(shape, c, *x, eps=1e-5, iflag=1, modeord=mo, single=True)
    assert a.dtype == np.complex64
    assert rel_l2(a, cn.nufft1(shape, c, *x, eps=1e-5, iflag=1, modeord=mo)) < 2e-6
    b = cn.nufft2(f, *x, eps=1e-5, iflag=-1, modeord=mo, single=True)
    assert b.dtype == np.complex64
    assert rel_l2(b, cn.nufft2(f, *x, eps=1e-5, iflag=-1, modeord=mo)) < 2e-6


@pytest.mark.parametrize("eps", [1e-3, 1e-5, 1e-6, 1e-9])
@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_kaiser_bessel_meets_eps(cn, eps, ndim):
    """The Kaiser-Bessel shape (gpu_kernel=1; beta of Beatty et al. 2005,
    the same width rule) against the direct sum: within eps at these sizes,
    and below the exponential of semicircle's error at the same width."""
    from oracle import direct

    rng = np.random.default_rng(20 + ndim)
    shape = {1: (30,), 2: (24, 31), 3: (20, 17, 24)}[ndim]
    x = [rng.uniform(-np.pi, np.pi, 3000) for _ in range(ndim)]
    f = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    exact = direct.type2(f, x, 1)
    e_kb = rel_l2(cn.nufft2(f, *x, eps=eps, iflag=1, kernel=1), exact)
    e_es = rel_l2(cn.nufft2(f, *x, eps=eps, iflag=1, kernel=0), exact)
    assert e_kb <= eps and e_kb < e_es, (e_kb, e_es)
    c = rng.normal(size=3000) + 1j * rng.normal(size=3000)
    assert rel_l2(cn.nufft1(shape, c, *x, eps=eps, iflag=1, kernel=1),
                  direct.type1(c, x, shape, 1)) <= eps
    s = [rng.uniform(-15, 15, 200) for _ in range(ndim)]
    assert rel_l2(cn.nufft3(c, *x, *s, eps=eps, iflag=1, kernel=1),
                  direct.type3(c, x, s, 1)) <= 2 * eps


def test_kaiser_bessel_meets_the_held_case(cn):
    """The one known answer the exponential of semicircle misses elementwise
    at width 11 (helpers.ORACLE_HELD) is met by Kaiser-Bessel at the same
    width."""
    g = golden("forward.npz")
    k = "t1_d3_x64_i-1"
    x, c, f = g[k + "_x"], g[k + "_c"], g[k + "_f"]
    check_reference(cn.nufft1(f.shape, c, *x, eps=1e-10, iflag=-1, kernel=1), f)


def test_kaiser_bessel_horner_fit(cn):
    """Degree w+2 piecewise polynomials reproduce the Kaiser-Bessel shape
    to ~1e-8 at w = 6 and to round-off from w = 10 (sigma = 2)."""
    for w, bound in ((4, 2e-5), (6, 5e-8), (8, 1e-10), (10, 1e-13), (13, 5e-14), (16, 5e-14)):
        _, beta, _ = cn.kernel_params(10.0 ** (1 - w), 2.0, 1)
        coef = cn.horner_fit(w, beta, w + 2, shape=1)
        d = np.linspace(0, 1, 257)[:-1]
        worst = 0.0
        for j in range(w):
            fit = np.polynomial.polynomial.polyval(2 * d - 1, coef[j])
            worst = max(worst, np.max(np.abs(fit - cn.kernel(j - w / 2 + d, w, beta, 1))))
        assert worst < bound, (w, worst)
