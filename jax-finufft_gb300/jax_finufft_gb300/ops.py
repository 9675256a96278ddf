"""nufft1 / nufft2 / nufft3 on GB300, with the reference's call signatures.

Mirrors src/jax_finufft/ops.py:
  * nufft1(output_shape, source, *points, iflag=1, eps=1e-6, opts=None)   (:50-82)
  * nufft2(source, *points, iflag=-1, eps=1e-6, opts=None)                (:85-111)
  * nufft3(source, *points, iflag=-1, eps=1e-6, opts=None)                (:126-155)
with the same broadcasting/flattening (shapes.py), the same forward-mode
rule (jvp, :158-277), reverse mode (the transpose rules of :280-314 written
as torch's conjugate-Wirtinger VJP) and the same vmap batching rule
(:317-353).  Tensors must live on a CUDA device; every transform runs in
libgbnufft.so through the C ABI (gbn_run) on the current torch stream.

Reverse mode, when a type-1/2 input requires grad, runs the fused adjoint:
the forward keeps its sorted point sets and the backward calls gbn_grad,
which builds the d+1 k-weighted grids in one pass, transforms them with one
batched cuFFT and gathers the strength gradient and every coordinate
gradient in a single interpolation pass on the forward's sort.  For type 3
(strengths and source points) the forward keeps its plans and the backward
is one adjoint pass on the same sorted sources and targets whose gather also
differentiates along the sources.  ``Opts(gpu_fused_adjoint=False)`` selects
the stacked-transform rules of the reference instead; so do gradients with
respect to type-3 targets.
"""
import threading

import numpy as np
import torch
import torch.autograd.forward_ad as _forward_ad

from . import _fused, _native, tune
from .options import Opts, to_native, unpack_opts
from .shapes import broadcast_and_flatten_inputs, check_canonical

# forward -> setup_context hand-off of a fused forward's point sets (torch
# calls the two back to back on the same thread)
_tls = threading.local()

__all__ = ["nufft1", "nufft2", "nufft3", "get_frequency_array"]


def get_frequency_array(n, modeord):
    """Integer frequencies of n modes in storage order (ops.py:114-123)."""
    if modeord == 0:
        return np.arange(-(n // 2), (n + 1) // 2)
    elif modeord == 1:
        f = np.empty(n, dtype=np.int64)
        f[: (n + 1) // 2] = np.arange(0, (n + 1) // 2)
        f[(n + 1) // 2:] = np.arange(-(n // 2), 0)
        return f
    raise ValueError(f"Unsupported modeord: {modeord}")


_DEFAULT_OPTS = Opts()

# gbn_opts structs of the options seen by _execute, by value (Opts is frozen;
# the structs are passed read-only to the library and never modified here)
_native_cache = {}


def _native_opts(fwd):
    n = _native_cache.get(fwd)
    if n is None:
        if len(_native_cache) > 64:
            _native_cache.clear()
        n = _native_cache[fwd] = to_native(fwd)
    return n


def _modeord(opts):
    return int(opts.modeord) if hasattr(opts, "modeord") else 0


def _execute(nufft_type, source, points, output_shape, iflag, eps, opts):
    """One native call on canonical buffers (see shapes.py)."""
    single = check_canonical(source, points, nufft_type)
    dev = source.device
    if dev.type != "cuda" or any(p.device != dev for p in points):
        raise RuntimeError("jax_finufft_gb300 runs on CUDA tensors only (all inputs on one "
                           "device); got %s" % ([str(dev)] + [str(p.device) for p in points]))
    ndim = len(points) // 2 if nufft_type == 3 else len(points)
    fwd = unpack_opts(opts, nufft_type, True)
    if fwd is None:
        fwd = _DEFAULT_OPTS
    n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
    n_j = int(points[0].shape[1])
    if nufft_type == 1:
        n_k = tuple(int(n) for n in output_shape)
        out_shape = (n_tot, n_transf) + n_k
        nk_b = list(n_k[::-1]) + [1] * (3 - ndim)
    elif nufft_type == 2:
        n_k = tuple(int(n) for n in source.shape[2:])
        out_shape = (n_tot, n_transf, n_j)
        nk_b = list(n_k[::-1]) + [1] * (3 - ndim)
    else:
        n_tgt = int(points[ndim].shape[1])
        out_shape = (n_tot, n_transf, n_tgt)
        nk_b = [n_tgt, 1, 1]
    out = torch.empty(out_shape, dtype=source.dtype, device=dev)
    if out.numel() == 0:
        return out
    if nufft_type in (1, 3) and n_j == 0:
        return out.zero_()
    src = source.contiguous()
    pts = [p.contiguous() for p in points[:ndim]][::-1]
    tgts = [p.contiguous() for p in points[ndim:]][::-1] if nufft_type == 3 else []
    eps_v = float(np.float32(eps)) if single else float(eps)
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev).cuda_stream
        native = _native_opts(fwd)
        if getattr(fwd, "gpu_autotune", False) and nufft_type in (1, 2):
            native, _ = tune.tuned_native(nufft_type, ndim, single, nk_b, n_j, n_transf, eps_v,
                                          int(iflag), native, stream)
        _native.run(nufft_type, ndim, single, stream, eps_v, int(iflag), n_tot, n_transf, n_j,
                    nk_b, native, src.data_ptr(), [p.data_ptr() for p in pts],
                    [p.data_ptr() for p in tgts], out.data_ptr())
    return out


def _freq_tensor(n, modeord, dim, ndim, like):
    """k along mode axis `dim` shaped to broadcast over (..., N_0, ..., N_{d-1})."""
    k = torch.as_tensor(get_frequency_array(int(n), modeord), device=like.device)
    k = k.to(torch.float32 if like.dtype == torch.complex64 else torch.float64)
    shape = [1] * ndim
    shape[dim] = -1
    return k.reshape(shape)


def _execute_fused(nufft_type, source, points, output_shape, iflag, eps, opts):
    """Forward that keeps its sorted point sets (types 1/2) or its plans
    (type 3) for the backward."""
    single = check_canonical(source, points, nufft_type)
    dev = source.device
    if dev.type != "cuda" or any(p.device != dev for p in points):
        raise RuntimeError("jax_finufft_gb300 runs on CUDA tensors only (all inputs on one "
                           "device); got %s" % ([str(dev)] + [str(p.device) for p in points]))
    if nufft_type == 3:
        ndim = len(points) // 2
        n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
        out = torch.empty((n_tot, n_transf, int(points[ndim].shape[1])), dtype=source.dtype,
                          device=dev)
        if out.numel() == 0 or source.numel() == 0 or int(points[0].shape[1]) == 0:
            return _execute(nufft_type, source, points, output_shape, iflag, eps, opts), None
        with torch.cuda.device(dev):
            state = _fused.t3_forward(source, points, iflag, eps, opts, out, single, ndim)
        return out, state
    ndim = len(points)
    n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
    n_j = int(points[0].shape[1])
    if nufft_type == 1:
        out_shape = (n_tot, n_transf) + tuple(int(n) for n in output_shape)
    else:
        out_shape = (n_tot, n_transf, n_j)
    out = torch.empty(out_shape, dtype=source.dtype, device=dev)
    if out.numel() == 0 or source.numel() == 0 or n_j == 0:
        return _execute(nufft_type, source, points, output_shape, iflag, eps, opts), None
    with torch.cuda.device(dev):
        state = _fused.forward(nufft_type, source, points, output_shape, iflag, eps, opts, out,
                               single, ndim)
    return out, state


def _wants_fused(nufft_type, opts, source, points):
    if not torch.is_grad_enabled():
        return False
    fwd = unpack_opts(opts, nufft_type, True)
    if fwd is not None and not getattr(fwd, "gpu_fused_adjoint", True):
        return False
    if nufft_type == 3:
        # strengths and sources only: target gradients take the stacked rules
        nd = len(points) // 2
        if any(p.requires_grad for p in points[nd:]):
            return False
    return bool(source.requires_grad or any(p.requires_grad for p in points))


def _no_transform_active(source, points):
    """True when nothing needs the autograd Function around a call: no input
    requires grad (or grad mode is off), no forward-mode dual level is open
    and no functorch transform (vmap, grad, jvp) is active.  The Function's
    machinery then costs more host time than a small transform's kernels;
    with an unknown torch the Function is always used."""
    if torch.is_grad_enabled() and (source.requires_grad
                                    or any(p.requires_grad for p in points)):
        return False
    level = getattr(_forward_ad, "_current_level", None)
    active = getattr(torch._C, "_are_functorch_transforms_active", None)
    if level is None or level != -1 or active is None:
        return False
    return not active()


def _apply(source, nufft_type, output_shape, iflag, eps, opts, fused, *points):
    if not fused and _no_transform_active(source, points):
        return _execute(nufft_type, source, points, output_shape, iflag, eps, opts)
    return _Nufft.apply(source, nufft_type, output_shape, iflag, eps, opts, fused, *points)


class _Nufft(torch.autograd.Function):
    """One canonical NUFFT call with its VJP, JVP and vmap rules."""

    @staticmethod
    def forward(source, nufft_type, output_shape, iflag, eps, opts, fused, *points):
        if fused:
            out, state = _execute_fused(nufft_type, source, points, output_shape, iflag, eps,
                                        opts)
            _tls.state = state
            return out
        _tls.state = None
        return _execute(nufft_type, source, points, output_shape, iflag, eps, opts)

    @staticmethod
    def setup_context(ctx, inputs, output):
        source, nufft_type, output_shape, iflag, eps, opts, fused, *points = inputs
        ctx.cfg = (nufft_type, output_shape, iflag, eps, opts)
        ctx.fused_state = getattr(_tls, "state", None) if fused else None
        _tls.state = None
        ctx.save_for_backward(source, *points)
        ctx.save_for_forward(source, *points)

    # --- reverse mode ------------------------------------------------------
    @staticmethod
    def backward(ctx, g):
        nufft_type, output_shape, iflag, eps, opts = ctx.cfg
        source, *points = ctx.saved_tensors
        need = ctx.needs_input_grad
        need_src = need[0]
        need_pts = list(need[7:])
        ndim = len(points) // 2 if nufft_type == 3 else len(points)
        if ctx.fused_state is not None and not torch.is_grad_enabled():
            # one fused adjoint on the forward's sort (not differentiable again:
            # a graph of the backward takes the stacked path below)
            with torch.cuda.device(source.device):
                if nufft_type == 3:
                    grad_src, gpts = _fused.t3_backward(ctx.fused_state, source, points, g,
                                                        need_src, need_pts)
                    gpts = gpts + [None] * ndim
                else:
                    grad_src, gpts = _fused.backward(ctx.fused_state, nufft_type, source,
                                                     points, g, need_src, need_pts)
            return (grad_src, None, None, None, None, None, None, *gpts)
        grads_pts = [None] * len(points)
        grad_src = None
        g = g.contiguous()
        n_tot, n_tr = source.shape[:2]
        if nufft_type == 1:
            # adjoint of type 1 is type 2 with -iflag; point terms weight g by k_d
            mo = _modeord(opts)
            dims = [d for d in range(ndim) if need_pts[d]]
            stack = ([g] if need_src else []) + [
                g * _freq_tensor(output_shape[d], mo, d, ndim, g) for d in dims]
            if stack:
                G = torch.stack(stack, dim=2).reshape((n_tot, n_tr * len(stack)) + tuple(g.shape[2:]))
                H = _Nufft.apply(G, 2, None, -iflag, eps, unpack_opts(opts, 2, False), False, *points)
                H = H.reshape(n_tot, n_tr, len(stack), -1)
                off = 0
                if need_src:
                    grad_src = H[:, :, 0]
                    off = 1
                for i, d in enumerate(dims):
                    grads_pts[d] = torch.real(
                        (1j * iflag) * source * torch.conj(H[:, :, off + i])).sum(dim=1)
        elif nufft_type == 2:
            mo = _modeord(opts)
            N = tuple(source.shape[2:])
            if need_src:
                grad_src = _Nufft.apply(g, 1, N, -iflag, eps, unpack_opts(opts, 1, False),
                                        False, *points)
            dims = [d for d in range(ndim) if need_pts[d]]
            if dims:
                stack = [(1j * iflag) * _freq_tensor(N[d], mo, d, ndim, source) * source
                         for d in dims]
                A = torch.stack(stack, dim=2).reshape((n_tot, n_tr * len(dims)) + N)
                H = _Nufft.apply(A, 2, None, iflag, eps, opts, False, *points)
                H = H.reshape(n_tot, n_tr, len(dims), -1)
                for i, d in enumerate(dims):
                    grads_pts[d] = torch.real(torch.conj(g) * H[:, :, i]).sum(dim=1)
        else:
            xs, ss = points[:ndim], points[ndim:]
            bopts = unpack_opts(opts, 3, False)
            dims_x = [d for d in range(ndim) if need_pts[d]]
            dims_s = [d for d in range(ndim) if need_pts[ndim + d]]
            stack = ([g] if need_src else []) + [g * ss[d][:, None, :] for d in dims_x]
            if stack:
                G = torch.stack(stack, dim=2).reshape(n_tot, n_tr * len(stack), -1)
                H = _Nufft.apply(G, 3, None, -iflag, eps, bopts, False, *ss, *xs)
                H = H.reshape(n_tot, n_tr, len(stack), -1)
                off = 0
                if need_src:
                    grad_src = H[:, :, 0]
                    off = 1
                for i, d in enumerate(dims_x):
                    grads_pts[d] = torch.real(
                        (1j * iflag) * source * torch.conj(H[:, :, off + i])).sum(dim=1)
            if dims_s:
                A = torch.stack([(1j * iflag) * xs[d][:, None, :] * source for d in dims_s],
                                dim=2).reshape(n_tot, n_tr * len(dims_s), -1)
                H2 = _Nufft.apply(A, 3, None, iflag, eps, opts, False, *xs, *ss)
                H2 = H2.reshape(n_tot, n_tr, len(dims_s), -1)
                for i, d in enumerate(dims_s):
                    grads_pts[ndim + d] = torch.real(torch.conj(g) * H2[:, :, i]).sum(dim=1)
        return (grad_src, None, None, None, None, None, None, *grads_pts)

    # --- forward mode (ops.py:158-277) ----------------------------------------
    @staticmethod
    def jvp(ctx, dsource, _t, _o, _i, _e, _p, _f, *dpoints):
        nufft_type, output_shape, iflag, eps, opts = ctx.cfg
        source, *points = ctx.saved_tensors
        ndim = len(points) // 2 if nufft_type == 3 else len(points)
        mo = _modeord(opts)
        n_tot, n_tr = source.shape[:2]
        out = None

        def add(a, b):
            return b if a is None else a + b

        if nufft_type == 1:
            args, scales = [], []
            if dsource is not None:
                args.append(dsource)
                scales.append(None)
            for d in range(ndim):
                if dpoints[d] is None:
                    continue
                args.append(dpoints[d][:, None, :] * source)
                scales.append((1j * iflag) * _freq_tensor(output_shape[d], mo, d, ndim, source))
            if args:
                R = _Nufft.apply(torch.stack(args, 2).reshape(n_tot, n_tr * len(args), -1), 1,
                                 output_shape, iflag, eps, opts, False, *points)
                R = R.reshape((n_tot, n_tr, len(args)) + tuple(output_shape))
                for i, s in enumerate(scales):
                    out = add(out, R[:, :, i] if s is None else s * R[:, :, i])
        elif nufft_type == 2:
            N = tuple(source.shape[2:])
            if dsource is not None:
                out = add(out, _Nufft.apply(dsource, 2, None, iflag, eps, opts, False, *points))
            dims = [d for d in range(ndim) if dpoints[d] is not None]
            if dims:
                A = torch.stack([(1j * iflag) * _freq_tensor(N[d], mo, d, ndim, source) * source
                                 for d in dims], 2).reshape((n_tot, n_tr * len(dims)) + N)
                R = _Nufft.apply(A, 2, None, iflag, eps, opts, False, *points)
                R = R.reshape(n_tot, n_tr, len(dims), -1)
                for i, d in enumerate(dims):
                    out = add(out, dpoints[d][:, None, :] * R[:, :, i])
        else:
            xs, ss = points[:ndim], points[ndim:]
            args, scales = [], []
            if dsource is not None:
                args.append(dsource)
                scales.append(None)
            for d in range(ndim):
                if dpoints[d] is None:
                    continue
                args.append(dpoints[d][:, None, :] * source)
                scales.append((1j * iflag) * ss[d][:, None, :])
            if args:
                R = _Nufft.apply(torch.stack(args, 2).reshape(n_tot, n_tr * len(args), -1), 3,
                                 None, iflag, eps, opts, False, *points)
                R = R.reshape(n_tot, n_tr, len(args), -1)
                for i, s in enumerate(scales):
                    out = add(out, R[:, :, i] if s is None else s * R[:, :, i])
            dims_s = [d for d in range(ndim) if dpoints[ndim + d] is not None]
            if dims_s:
                A = torch.stack([(1j * iflag) * xs[d][:, None, :] * source for d in dims_s],
                                2).reshape(n_tot, n_tr * len(dims_s), -1)
                R = _Nufft.apply(A, 3, None, iflag, eps, opts, False, *points)
                R = R.reshape(n_tot, n_tr, len(dims_s), -1)
                for i, d in enumerate(dims_s):
                    out = add(out, dpoints[ndim + d][:, None, :] * R[:, :, i])
        if out is None:
            out = torch.zeros_like(_execute(nufft_type, source, points, output_shape, iflag,
                                            eps, opts))
        return out

    # --- vmap (ops.py:317-353) -------------------------------------------------
    @staticmethod
    def vmap(info, in_dims, source, nufft_type, output_shape, iflag, eps, opts, fused, *points):
        sdim = in_dims[0]
        pdims = in_dims[7:]
        B = info.batch_size
        if all(d is None for d in pdims):
            # unmapped points: one transform stack of n_transf * B
            src = source.movedim(sdim, 0)
            n_tot, n_tr = src.shape[1], src.shape[2]
            src = src.movedim(0, 1).reshape((n_tot, B * n_tr) + tuple(src.shape[3:]))
            out = _Nufft.apply(src, nufft_type, output_shape, iflag, eps, opts, fused, *points)
            out = out.reshape((n_tot, B, n_tr) + tuple(out.shape[2:]))
            return out, 1
        src = source.movedim(sdim, 0) if sdim is not None else source.unsqueeze(0).expand(
            (B,) + tuple(source.shape))
        pts = [p.movedim(d, 0) if d is not None else p.unsqueeze(0).expand((B,) + tuple(p.shape))
               for p, d in zip(points, pdims)]
        n_tot = src.shape[1]
        src = src.reshape((B * n_tot,) + tuple(src.shape[2:]))
        pts = [p.reshape((B * n_tot,) + tuple(p.shape[2:])) for p in pts]
        out = _Nufft.apply(src, nufft_type, output_shape, iflag, eps, opts, fused, *pts)
        return out.reshape((B, n_tot) + tuple(out.shape[1:])), 0


def nufft1(output_shape, source, *points, iflag=1, eps=1e-6, opts=None):
    """Type 1: f_k = sum_j c_j exp(iflag*i*k.x_j), modes per ``output_shape``."""
    iflag = int(iflag)
    eps = float(eps)
    ndim = len(points)
    if not 1 <= ndim <= 3:
        raise ValueError("Only 1-, 2-, and 3-dimensions are supported")
    output_shape = np.atleast_1d(output_shape).astype(np.int64)
    if output_shape.shape != (ndim,):
        raise ValueError(f"output_shape must have shape: ({ndim},)")
    output_shape = tuple(int(n) for n in output_shape)
    index, source, *points = broadcast_and_flatten_inputs(1, output_shape, source, *points)
    fused = _wants_fused(1, opts, source, points)
    result = _apply(source, 1, output_shape, iflag, eps, opts, fused, *points)
    return index.unflatten(result)


def nufft2(source, *points, iflag=-1, eps=1e-6, opts=None):
    """Type 2: c_j = sum_k f_k exp(iflag*i*k.x_j)."""
    iflag = int(iflag)
    eps = float(eps)
    ndim = len(points)
    if not 1 <= ndim <= 3:
        raise ValueError("Only 1-, 2-, and 3-dimensions are supported")
    index, source, *points = broadcast_and_flatten_inputs(2, None, source, *points)
    fused = _wants_fused(2, opts, source, points)
    result = _apply(source, 2, None, iflag, eps, opts, fused, *points)
    return index.unflatten(result)


def nufft3(source, *points, iflag=-1, eps=1e-6, opts=None):
    """Type 3: f_k = sum_j c_j exp(iflag*i*s_k.x_j); points = sources..., targets...."""
    iflag = int(iflag)
    eps = float(eps)
    twice_ndim = len(points)
    if twice_ndim % 2 != 0:
        raise ValueError("nufft3 requires an even number of point arrays")
    ndim = twice_ndim // 2
    if not 1 <= ndim <= 3:
        raise ValueError("Only 1-, 2-, and 3-dimensions are supported")
    index, source, *points = broadcast_and_flatten_inputs(3, None, source, *points)
    fused = _wants_fused(3, opts, source, points)
    result = _apply(source, 3, None, iflag, eps, opts, fused, *points)
    return index.unflatten(result)
