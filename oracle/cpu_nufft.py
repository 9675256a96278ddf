"""CPU restatement of the fast NUFFT -- test infrastructure only.

Restates the algorithm of the vendored (absent) FINUFFT/cuFINUFFT that
lib/kernels.cc.cu:25-92 drives through makeplan/setpts/execute:
  type 1: fold + bin  ->  spread with the ES kernel  ->  FFT on the
          upsampled grid  ->  deconvolve by the kernel's Fourier transform and
          reorder modes (modeord, src/jax_finufft/ops.py:114-123);
  type 2: deconvolve + zero-pad  ->  FFT  ->  interpolate;
  type 3: rescale, pre-phase, spread, inner type 2, post-phase/deconvolve.
The per-point arithmetic (fold, grid start, kernel values, spread, interp) is
the C code in nufft_oracle.c; the FFT is numpy/scipy pocketfft; all in FP64.

Axes are in the user's order (point array ``a`` pairs with mode axis ``a``);
the C code receives them reversed, as lowering.py:96-105 does for the backend.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from .direct import frequencies

try:  # scipy's pocketfft takes a thread count; numpy's does not
    import scipy.fft as _sfft
except Exception:  # pragma: no cover - scipy is on both machines
    _sfft = None

_LIB = None
_i64p = ctypes.POINTER(ctypes.c_int64)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def lib():
    """Load (building on first use) the oracle's C library."""
    global _LIB
    if _LIB is None:
        path = _build.library_path()
        if not os.path.exists(path):
            _build.build()
        L = ctypes.CDLL(path)
        L.orc_next235even.restype = ctypes.c_int64
        L.orc_next235even.argtypes = [ctypes.c_int64]
        L.orc_kernel_params.restype = ctypes.c_int
        L.orc_kernel_params.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _ip, _dp]
        L.orc_fine_size.restype = ctypes.c_int64
        L.orc_fine_size.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_int]
        L.orc_kernel.restype = ctypes.c_double
        L.orc_kernel.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_kernel_ft.restype = None
        L.orc_kernel_ft.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int64,
                                    _dp, _dp]
        L.orc_fold.restype = ctypes.c_double
        L.orc_fold.argtypes = [ctypes.c_double, ctypes.c_int64]
        L.orc_fold_points.restype = None
        L.orc_fold_points.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i64p, _ip,
                                      ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _i64p, _dp,
                                      _i64p]
        L.orc_spread.restype = None
        L.orc_spread.argtypes = [ctypes.c_int, _i64p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_int64, _i64p, _dp, _dp, _dp]
        L.orc_interp.restype = None
        L.orc_interp.argtypes = [ctypes.c_int, _i64p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_int64, _i64p, _dp, _dp, _dp]
        _fp = ctypes.POINTER(ctypes.c_float)
        for name in ("orc_spread_f32", "orc_interp_f32"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [ctypes.c_int, _i64p, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int64,
                           _i64p, _fp, _fp, _fp]
        L.orc_deconv_f32.restype = None
        L.orc_deconv_f32.argtypes = [ctypes.c_int, ctypes.c_int, _i64p, _i64p, _i64p, _i64p,
                                     _i64p, _fp, _fp, _fp, _fp, _fp]
        L.orc_horner_fit.restype = None
        L.orc_horner_fit.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                     _dp]
        L.orc_type3_params.restype = ctypes.c_int64
        L.orc_type3_params.argtypes = [ctypes.c_double] * 5 + [ctypes.c_int, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


def set_threads(n):
    lib().orc_set_threads(int(n))


def num_threads():
    return int(lib().orc_num_threads())


# --------------------------------------------------------------------------
# plan-time parameters
# --------------------------------------------------------------------------

def kernel_params(eps, sigma=2.0, shape=0):
    """(w, beta, warn) for tolerance eps at upsampling factor sigma; shape 0
    the exponential of semicircle, 1 Kaiser-Bessel."""
    w = ctypes.c_int()
    b = ctypes.c_double()
    warn = lib().orc_kernel_params(float(eps), float(sigma), int(shape), ctypes.byref(w),
                                   ctypes.byref(b))
    return w.value, b.value, int(warn)


def fine_size(n, sigma, w):
    return int(lib().orc_fine_size(int(n), float(sigma), int(w)))


def next235even(n):
    return int(lib().orc_next235even(int(n)))


def kernel(t, w, beta, shape=0):
    return np.array([lib().orc_kernel(float(x), int(w), float(beta), int(shape))
                     for x in np.ravel(t)])


def kernel_ft(w, beta, omega, shape=0):
    om = np.ascontiguousarray(np.ravel(omega), dtype=np.float64)
    out = np.empty_like(om)
    lib().orc_kernel_ft(int(w), float(beta), int(shape), om.size, _p(om, _dp), _p(out, _dp))
    return out.reshape(np.shape(omega))


def horner_fit(w, beta, deg, shape=0):
    coef = np.empty(w * (deg + 1))
    lib().orc_horner_fit(int(w), float(beta), int(shape), int(deg), _p(coef, _dp))
    return coef.reshape(w, deg + 1)


def type3_params(xmin, xmax, smin, smax, sigma, w):
    out = np.empty(3)
    nf = lib().orc_type3_params(float(xmin), float(xmax), float(smin), float(smax), float(sigma),
                                int(w), _p(out, _dp))
    return int(nf), float(out[0]), float(out[1]), float(out[2])


def fold_points(coords_b, nf_b, w, binsize_b=(1, 1, 1), mode=0, center_b=None, scale_b=None):
    """Per-point fold in backend order (x fastest).

    Returns (X, i0, delta, bin) with X/i0/delta of shape (M, 3) and bin (M,).
    ``mode`` 0 folds periodically; 1 applies the type-3 rescale with
    ``center_b``/``scale_b``.
    """
    dim = len(coords_b)
    cs = [np.ascontiguousarray(c, dtype=np.float64) for c in coords_b]
    M = cs[0].shape[0]
    while len(cs) < 3:
        cs.append(cs[0])
    nf = np.ones(3, dtype=np.int64)
    nf[:dim] = nf_b
    bs = np.ones(4, dtype=np.int32)
    bs[:3] = list(binsize_b) + [1] * (3 - len(binsize_b))
    cen = np.zeros(3)
    sc = np.ones(3)
    if center_b is not None:
        cen[:dim] = center_b
        sc[:dim] = scale_b
    X = np.empty((M, 3))
    i0 = np.empty((M, 3), dtype=np.int64)
    de = np.empty((M, 3))
    b = np.empty(M, dtype=np.int64)
    lib().orc_fold_points(dim, int(mode), int(w), _p(nf, _i64p), bs.ctypes.data_as(_ip), M,
                          _p(cs[0], _dp), _p(cs[1], _dp), _p(cs[2], _dp), _p(cen, _dp),
                          _p(sc, _dp), _p(X, _dp), _p(i0, _i64p), _p(de, _dp), _p(b, _i64p))
    return X, i0, de, b


def _spread(nf_b, w, beta, i0, de, c, shape=0):
    dim = len(nf_b)
    nf = np.ones(3, dtype=np.int64)
    nf[:dim] = nf_b
    grid = np.zeros(int(np.prod(nf_b)), dtype=np.complex128)
    cc = np.ascontiguousarray(c, dtype=np.complex128)
    lib().orc_spread(dim, _p(nf, _i64p), int(w), float(beta), int(shape), cc.shape[0],
                     _p(i0, _i64p),
                     _p(de, _dp), cc.view(np.float64).ctypes.data_as(_dp),
                     grid.view(np.float64).ctypes.data_as(_dp))
    return grid.reshape(tuple(nf_b[::-1]))


def _interp(nf_b, w, beta, i0, de, grid, shape=0):
    dim = len(nf_b)
    nf = np.ones(3, dtype=np.int64)
    nf[:dim] = nf_b
    g = np.ascontiguousarray(grid, dtype=np.complex128).ravel()
    M = i0.shape[0]
    out = np.empty(M, dtype=np.complex128)
    lib().orc_interp(dim, _p(nf, _i64p), int(w), float(beta), int(shape), M, _p(i0, _i64p),
                     _p(de, _dp),
                     g.view(np.float64).ctypes.data_as(_dp),
                     out.view(np.float64).ctypes.data_as(_dp))
    return out


def _fft(grid, iflag, workers):
    """Unnormalised FFT with exponent sign iflag over all axes."""
    axes = tuple(range(grid.ndim))
    if _sfft is not None:
        if iflag >= 0:
            return _sfft.ifftn(grid, axes=axes, norm="forward", workers=workers)
        return _sfft.fftn(grid, axes=axes, workers=workers)
    if iflag >= 0:
        return np.fft.ifftn(grid, axes=axes) * grid.size
    return np.fft.fftn(grid, axes=axes)


def _workers():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:  # pragma: no cover
        return os.cpu_count() or 1


class Plan:
    """Plan-time quantities for types 1/2 in the user's axis order."""

    def __init__(self, n_modes, eps, sigma=2.0, modeord=0, kernel=0):
        self.n_modes = tuple(int(n) for n in n_modes)
        self.dim = len(self.n_modes)
        self.shape = int(kernel)
        self.w, self.beta, self.warn = kernel_params(eps, sigma, self.shape)
        self.sigma = sigma
        self.modeord = modeord
        self.nf = tuple(fine_size(n, sigma, self.w) for n in self.n_modes)
        self.ks = [frequencies(n, modeord) for n in self.n_modes]
        self.idx = [np.mod(k, nf) for k, nf in zip(self.ks, self.nf)]
        self.phihat = [kernel_ft(self.w, self.beta, 2 * np.pi * k / nf, self.shape)
                       for k, nf in zip(self.ks, self.nf)]

    def deconv_factor(self):
        f = np.ones((), dtype=np.float64)
        for ph in self.phihat:
            f = np.multiply.outer(f, 1.0 / ph)
        return f

    def fold(self, points):
        X, i0, de, b = fold_points(list(points)[::-1], list(self.nf)[::-1], self.w)
        return i0, de


def _f32_args(plan, i0, de):
    """Arguments of the single-precision C routines for plan's geometry."""
    deg = plan.w + 2
    coef = np.ascontiguousarray(horner_fit(plan.w, plan.beta, deg, plan.shape).ravel())
    nf = np.ones(3, dtype=np.int64)
    nf[:plan.dim] = list(plan.nf)[::-1]
    return (plan.dim, _p(nf, _i64p), plan.w, deg, _p(coef, _dp), i0.shape[0], _p(i0, _i64p),
            _p(np.ascontiguousarray(de, dtype=np.float32), ctypes.POINTER(ctypes.c_float))), \
        (nf, coef, de)


def _spread_f32(plan, i0, de, c):
    args, keep = _f32_args(plan, i0, de)
    de32 = np.ascontiguousarray(de, dtype=np.float32)
    cc = np.ascontiguousarray(c, dtype=np.complex64)
    grid = np.zeros(int(np.prod(plan.nf)), dtype=np.complex64)
    fp = ctypes.POINTER(ctypes.c_float)
    lib().orc_spread_f32(*args[:7], _p(de32, fp), cc.view(np.float32).ctypes.data_as(fp),
                         grid.view(np.float32).ctypes.data_as(fp))
    return grid.reshape(plan.nf)


def _interp_f32(plan, i0, de, grid):
    args, keep = _f32_args(plan, i0, de)
    de32 = np.ascontiguousarray(de, dtype=np.float32)
    g = np.ascontiguousarray(grid, dtype=np.complex64).ravel()
    out = np.empty(i0.shape[0], dtype=np.complex64)
    fp = ctypes.POINTER(ctypes.c_float)
    lib().orc_interp_f32(*args[:7], _p(de32, fp), g.view(np.float32).ctypes.data_as(fp),
                         out.view(np.float32).ctypes.data_as(fp))
    return out


def _deconv_f32(plan, direction, f, grid):
    """Single-precision deconvolution between modes f and the fine grid
    (direction 1: zero-pad into grid; -1: crop into f), in C with threads."""
    fp = ctypes.POINTER(ctypes.c_float)
    rev = list(range(plan.dim))[::-1]  # backend order: the user's last axis first
    n = np.array([plan.n_modes[a] for a in rev] + [1] * (3 - plan.dim), dtype=np.int64)
    nf = np.array([plan.nf[a] for a in rev] + [1] * (3 - plan.dim), dtype=np.int64)
    idx = [np.ascontiguousarray(plan.idx[a], dtype=np.int64) for a in rev]
    fac = [np.ascontiguousarray(1.0 / plan.phihat[a], dtype=np.float32) for a in rev]
    while len(idx) < 3:
        idx.append(np.zeros(1, dtype=np.int64))
        fac.append(np.ones(1, dtype=np.float32))
    lib().orc_deconv_f32(direction, plan.dim, _p(n, _i64p), _p(nf, _i64p),
                         *[_p(i, _i64p) for i in idx], *[_p(a, fp) for a in fac],
                         f.view(np.float32).ctypes.data_as(fp),
                         grid.view(np.float32).ctypes.data_as(fp))


def nufft1(n_modes, c, *points, eps=1e-6, iflag=1, modeord=0, sigma=2.0, workers=None,
           single=False, kernel=0):
    """Type 1 in the user's axis order.  c: (M,) or (T, M) complex.

    single=True runs the single-precision fast path (complex64 throughout,
    kernel by Horner's rule, bin-sorted private subgrids): the timed CPU
    baseline, not the checker.  kernel: 0 the exponential of semicircle, 1
    Kaiser-Bessel."""
    workers = workers or _workers()
    plan = Plan(n_modes, eps, sigma, modeord, kernel)
    if single:
        i0, de = plan.fold(points)
        cs = np.asarray(c)
        cs = cs[None] if cs.ndim == 1 else cs
        out = np.empty((cs.shape[0],) + plan.n_modes, dtype=np.complex64)
        for t in range(cs.shape[0]):
            B = np.ascontiguousarray(_fft(_spread_f32(plan, i0, de, cs[t]), iflag, workers),
                                     dtype=np.complex64)
            _deconv_f32(plan, -1, out[t], B)
        return out[0] if np.asarray(c).ndim == 1 else out
    c = np.asarray(c)
    single = c.ndim == 1
    cs = c[None] if single else c
    i0, de = plan.fold(points)
    fac = plan.deconv_factor()
    outs = []
    for t in range(cs.shape[0]):
        grid = _spread(list(plan.nf)[::-1], plan.w, plan.beta, i0, de, cs[t], plan.shape)
        B = _fft(grid, iflag, workers)
        outs.append(B[np.ix_(*plan.idx)] * fac)
    out = np.stack(outs)
    return out[0] if single else out


def nufft2(f, *points, eps=1e-6, iflag=-1, modeord=0, sigma=2.0, workers=None, single=False,
           kernel=0):
    """Type 2 in the user's axis order.  f: (N...) or (T, N...) complex.
    single=True: the single-precision fast path (see nufft1)."""
    workers = workers or _workers()
    d = len(points)
    f = np.asarray(f)
    one = f.ndim == d
    fs = f[None] if one else f
    plan = Plan(fs.shape[1:], eps, sigma, modeord, kernel)
    i0, de = plan.fold(points)
    outs = []
    if single:
        grid = np.empty(plan.nf, dtype=np.complex64)
        for t in range(fs.shape[0]):
            _deconv_f32(plan, 1, np.ascontiguousarray(fs[t], dtype=np.complex64), grid)
            outs.append(_interp_f32(plan, i0, de, _fft(grid, iflag, workers)))
        out = np.stack(outs)
        return out[0] if one else out
    fac = plan.deconv_factor()
    for t in range(fs.shape[0]):
        grid = np.zeros(plan.nf, dtype=np.complex128)
        grid[np.ix_(*plan.idx)] = fs[t] * fac
        b = _fft(grid, iflag, workers)
        outs.append(_interp(list(plan.nf)[::-1], plan.w, plan.beta, i0, de, b, plan.shape))
    out = np.stack(outs)
    return out[0] if one else out


def type3_setup(sources, targets, eps, sigma=2.0, kernel=0):
    """Per-dimension type-3 parameters in the user's axis order."""
    w, beta, warn = kernel_params(eps, sigma, kernel)
    prm = []
    for x, s in zip(sources, targets):
        x = np.asarray(x, dtype=np.float64)
        s = np.asarray(s, dtype=np.float64)
        prm.append(type3_params(x.min(), x.max(), s.min(), s.max(), sigma, w))
    return w, beta, prm


def nufft3(c, *points, eps=1e-6, iflag=-1, sigma=2.0, workers=None, kernel=0):
    """Type 3 in the user's axis order: points = sources..., targets...."""
    workers = workers or _workers()
    d = len(points) // 2
    xs = [np.asarray(p, dtype=np.float64) for p in points[:d]]
    ss = [np.asarray(p, dtype=np.float64) for p in points[d:]]
    c = np.asarray(c)
    single = c.ndim == 1
    cs = c[None] if single else c
    w, beta, prm = type3_setup(xs, ss, eps, sigma, kernel)
    nf = [p[0] for p in prm]
    cen = [p[1] for p in prm]
    tcen = [p[2] for p in prm]
    scale = [p[3] for p in prm]
    # sources onto the spreading grid (backend order for the C code)
    X, i0, de, _ = fold_points(xs[::-1], nf[::-1], w, mode=1, center_b=cen[::-1],
                               scale_b=scale[::-1])
    # pre-phase with the target centre, post-phase with the source centre
    pre = np.exp(1j * iflag * sum(tc * (x - cc) for tc, x, cc in zip(tcen, xs, cen)))
    taus = [(s - tc) / sc for s, tc, sc in zip(ss, tcen, scale)]
    post = np.exp(1j * iflag * sum(cc * s for cc, s in zip(cen, ss)))
    for a in range(d):
        post = post / kernel_ft(w, beta, taus[a], kernel)
    outs = []
    for t in range(cs.shape[0]):
        grid = _spread(nf[::-1], w, beta, i0, de, cs[t] * pre, kernel)
        inner = nufft2(grid, *taus, eps=eps, iflag=iflag, modeord=0, sigma=sigma,
                       workers=workers, kernel=kernel)
        outs.append(inner * post)
    out = np.stack(outs)
    return out[0] if single else out
