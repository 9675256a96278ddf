"""The 18 reference-shaped entry points against the reference's known answers.

gbn_nufft{1,2,3}d{1,2,3}{f,} are what a jax-finufft FFI handler calls in
place of nufft{D}d{T}{f}_impl (lib/kernels.h:24-180).  Each test calls one
through ctypes exactly as src/jax_finufft/lowering.py:79-178 and
lib/jax_finufft_gpu.cc:28-60 would: the scalar attributes in the handler's
order, n_k_full = the user's mode shape reversed and zero-padded to three
entries (type 3: n_k_1 = number of targets, n_k_2 = n_k_3 = 0), the point
arrays in reversed user order, float32 eps for the ``f`` targets.

Expected values are the reference tests' own direct sums
(tests/golden/from_reference.py replays tests/ops_test.py:25-125).  The
comparison is the reference's check_close (ops_test.py:14-16: rtol 1e-7
complex128, 1e-4 complex64, 1e-3 for type-3 complex64; jax's default atol
1e-15 / 1e-6) elementwise, with no absolute floor.

One case is held to a different bar (helpers.ORACLE_HELD): 3D type 1,
float64, iflag -1 at eps 1e-10, where one of 26,250 modes misses the
elementwise bound even for the FP64 oracle with the exact kernel.  There the
entry point must come within 1.5x of the oracle's own per-entry error, and
the relative l2 bound still applies.
"""
import ctypes
from itertools import product

import numpy as np
import pytest
import torch

from helpers import ORACLE_HELD, check_reference, golden

pytestmark = pytest.mark.gpu

DEV = "cuda"
_vp = ctypes.c_void_p


def T(a):
    return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


def ptr(t):
    return _vp(t.data_ptr())


def attrs(x64, eps, iflag, n_tot, n_transf, n_j, n_k_full, modeord=0):
    """The handler's scalar attributes in jax_finufft_gpu.cc:28-60's order."""
    stream = _vp(torch.cuda.current_stream().cuda_stream)
    e = ctypes.c_double(eps) if x64 else ctypes.c_float(np.float32(eps))
    return [stream, e, iflag, n_tot, n_transf, n_j, int(n_k_full[0]), int(n_k_full[1]),
            int(n_k_full[2]), modeord, ctypes.c_double(2.0), 0, 1, 1, 0, 0]


def call(native, ty, ndim, x64, args, tensors):
    name = "gbn_nufft%dd%d%s" % (ndim, ty, "" if x64 else "f")
    rc = getattr(native, name)(*args, *[ptr(t) for t in tensors])
    torch.cuda.synchronize()
    assert rc == 0, (name, rc, native.gbn_last_error())


def n_k_full(shape):
    """lowering.py:96-100: the mode shape reversed, zero-padded to three."""
    nk = [0, 0, 0]
    nk[:len(shape)] = list(shape)[::-1]
    return nk


def run_type1(native, x64, iflag, eps, c, x, shape, n_tot=1, n_transf=1, modeord=0):
    """c: (n_tot, n_transf, M), x: (ndim, n_tot, M) in user order."""
    ndim = len(shape)
    M = c.shape[-1]
    out = torch.empty((n_tot, n_transf) + tuple(shape),
                      dtype=torch.complex128 if x64 else torch.complex64, device=DEV)
    pts = [T(x[d]) for d in range(ndim)][::-1]  # lowering.py:105
    call(native, 1, ndim, x64, attrs(x64, eps, iflag, n_tot, n_transf, M, n_k_full(shape),
                                     modeord), [T(c)] + pts + [out])
    return out.cpu().numpy()


def run_type2(native, x64, iflag, eps, f, x, n_tot=1, n_transf=1, modeord=0):
    """f: (n_tot, n_transf, N...), x: (ndim, n_tot, M)."""
    shape = f.shape[2:]
    ndim = len(shape)
    M = x.shape[-1]
    out = torch.empty((n_tot, n_transf, M), dtype=torch.complex128 if x64 else torch.complex64,
                      device=DEV)
    pts = [T(x[d]) for d in range(ndim)][::-1]
    call(native, 2, ndim, x64, attrs(x64, eps, iflag, n_tot, n_transf, M, n_k_full(shape),
                                     modeord), [T(f)] + pts + [out])
    return out.cpu().numpy()


def run_type3(native, x64, iflag, eps, c, x, s, n_tot=1, n_transf=1):
    """c: (n_tot, n_transf, M), x: (ndim, n_tot, M), s: (ndim, n_tot, N)."""
    ndim = x.shape[0]
    M, N = x.shape[-1], s.shape[-1]
    out = torch.empty((n_tot, n_transf, N), dtype=torch.complex128 if x64 else torch.complex64,
                      device=DEV)
    pts = [T(x[d]) for d in range(ndim)][::-1] + [T(s[d]) for d in range(ndim)][::-1]
    call(native, 3, ndim, x64, attrs(x64, eps, iflag, n_tot, n_transf, M, [N, 0, 0]),
         [T(c)] + pts + [out])
    return out.cpu().numpy()


FWD = list(product([1, 2, 3], [False, True], [-1, 1]))


def _key(ndim, x64, iflag):
    return "d%d_%s_i%+d" % (ndim, "x64" if x64 else "x32", iflag)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_named_type1(native, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t1_" + _key(ndim, x64, iflag)
    x, c, f = g[k + "_x"], g[k + "_c"], g[k + "_f"]
    eps = 1e-10 if x64 else 1e-7
    out = run_type1(native, x64, iflag, eps, c[None, None], x[:, None], f.shape)[0, 0]
    held = None
    if (1, ndim, x64, iflag) in ORACLE_HELD:
        from oracle import cpu_nufft

        held = cpu_nufft.nufft1(f.shape, c, *x, eps=eps, iflag=iflag)
    check_reference(out, f, held=held)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_named_type2(native, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t2_" + _key(ndim, x64, iflag)
    x, f, c = g[k + "_x"], g[k + "_f"], g[k + "_c"]
    eps = 1e-10 if x64 else 1e-7
    out = run_type2(native, x64, iflag, eps, f[None, None], x[:, None])[0, 0]
    check_reference(out, c)


@pytest.mark.parametrize("ndim, x64, iflag", FWD)
def test_named_type3(native, ndim, x64, iflag):
    g = golden("forward.npz")
    k = "t3_" + _key(ndim, x64, iflag)
    x, s, c, f = g[k + "_x"], g[k + "_s"], g[k + "_c"], g[k + "_f"]
    eps = 1e-10 if x64 else 1e-7
    out = run_type3(native, x64, iflag, eps, c[None, None], x[:, None], s[:, None])[0, 0]
    rtol = float(g["t3_rtol_complex128"] if x64 else g["t3_rtol_complex64"])
    check_reference(out, f, rtol=rtol)


@pytest.mark.parametrize("mo, nf, ndim, ty",
                         list(product([0, 1], [16, 17], [1, 2, 3], [1, 2])))
def test_named_modeord(native, mo, nf, ndim, ty):
    """test_modeord (ops_test.py:494-567) through the named entry points."""
    g = golden("modeord.npz")
    k = "mo%d_n%d_d%d_t%d" % (mo, nf, ndim, ty)
    x = g[k + "_x"]
    if ty == 1:
        c, f = g[k + "_c"], g[k + "_f"]
        out = run_type1(native, True, 1, 1e-10, c[None, None], x[:, None], f.shape,
                        modeord=mo)[0, 0]
        check_reference(out, f)
    else:
        f, c = g[k + "_f"], g[k + "_c"]
        out = run_type2(native, True, 1, 1e-10, f[None, None], x[:, None], modeord=mo)[0, 0]
        check_reference(out, c)


def test_named_n_tot(native):
    """n_tot = 5 independent point sets in one call (test_multi_transform,
    ops_test.py:380-397; run_nufft's offsets, lib/kernels.cc.cu:57-66)."""
    g = golden("multi.npz")
    n_k = int(g["n_k"])
    x = g["x"][None]  # (1, n_tot, M)
    n_tot, n_tr = g["c"].shape[:2]
    o1 = run_type1(native, True, 1, 1e-6, g["c"], x, (n_k,), n_tot=n_tot, n_transf=n_tr)
    o2 = run_type2(native, True, -1, 1e-6, g["f"], x, n_tot=n_tot, n_transf=n_tr)
    o3 = run_type3(native, True, -1, 1e-6, g["c"], x, g["xt"][None], n_tot=n_tot,
                   n_transf=n_tr)
    for out, exp in ((o1, g["t1"]), (o2, g["t2"]), (o3, g["t3"])):
        check_reference(out, exp, rtol=1e-4)
    # and each slice alone equals its row of the n_tot call
    for i in range(n_tot):
        one = run_type1(native, True, 1, 1e-6, g["c"][i:i + 1], x[:, i:i + 1], (n_k,))
        check_reference(one[0], o1[i], rtol=1e-4)


@pytest.mark.parametrize("ty, ndim, x64", list(product([1, 2, 3], [1, 2, 3], [False, True])))
def test_named_n_transf_and_n_tot(native, ty, ndim, x64):
    """n_transf = 3 stacked transforms sharing points, for n_tot = 2 point
    sets: strengths (or modes) c, (1+2i) c and -i c of the known-answer
    case, so the expected outputs are the known answer scaled (linearity)."""
    g = golden("forward.npz")
    k = "t%d_" % ty + _key(ndim, x64, 1)
    eps = 1e-10 if x64 else 1e-7
    scale = np.array([1.0, 1.0 + 2.0j, -1.0j])
    cd = np.complex128 if x64 else np.complex64
    if ty == 1:
        x, c, f = g[k + "_x"], g[k + "_c"], g[k + "_f"]
        src = (scale[:, None] * c[None]).astype(cd)
        src = np.stack([src, src[::-1]])  # point set 2 = same points, transforms reversed
        out = run_type1(native, x64, 1, eps, src, np.stack([x, x], axis=1), f.shape,
                        n_tot=2, n_transf=3)
        exp = (scale.reshape((3,) + (1,) * ndim) * f[None]).astype(cd)
    elif ty == 2:
        x, f, c = g[k + "_x"], g[k + "_f"], g[k + "_c"]
        src = (scale.reshape((3,) + (1,) * ndim) * f[None]).astype(cd)
        src = np.stack([src, src[::-1]])
        out = run_type2(native, x64, 1, eps, src, np.stack([x, x], axis=1), n_tot=2, n_transf=3)
        exp = (scale[:, None] * c[None]).astype(cd)
    else:
        x, s, c, f = g[k + "_x"], g[k + "_s"], g[k + "_c"], g[k + "_f"]
        src = (scale[:, None] * c[None]).astype(cd)
        src = np.stack([src, src[::-1]])
        out = run_type3(native, x64, 1, eps, src, np.stack([x, x], axis=1),
                        np.stack([s, s], axis=1), n_tot=2, n_transf=3)
        exp = (scale[:, None] * f[None]).astype(cd)
    rtol = None if ty != 3 else float(g["t3_rtol_complex128"] if x64 else g["t3_rtol_complex64"])
    for t in range(3):
        check_reference(out[0, t], exp[t], rtol=rtol)
        check_reference(out[1, t], exp[2 - t], rtol=rtol)
