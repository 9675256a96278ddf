"""Forward passes that keep their sorted points for a fused backward.

When a type-1 or type-2 transform may be differentiated, the forward sorts
each point set into a ``gbn_points`` object (one per n_tot index) and keeps
it; the backward hands the same point sets to ``gbn_grad``, which computes the
strength/mode gradient and every coordinate gradient with one batched cuFFT
of the stacked k-weighted grids and one interpolation pass.  The reference
instead issues separate transforms from its JVP and transpose rules
(src/jax_finufft/ops.py:158-314), each sorting the points again.

Plans (kernel coefficients, deconvolution factors, grids, cuFFT plans) are
cached here per (type, shape, options, precision, device, stream).
"""
import ctypes
import threading
from collections import OrderedDict

import numpy as np
import torch

from . import _native
from .options import Opts, to_native, unpack_opts

_lock = threading.Lock()
_plans = OrderedDict()  # key -> (plan handle, lock serialising its calls), most recent last
_MAX_PLANS = 8


def _opts_key(n):
    return tuple(getattr(n, f) for f, _ in n._fields_)


def get_plan(key):
    """(plan handle, lock) for a cache key (created on first use).  Threads
    that share a key share the plan; they hold its lock around every call
    on it (a plan's cuFFT handles and buffers serve one call at a time)."""
    lib = _native.load()
    with _lock:
        h = _plans.get(key)
        if h is not None:
            _plans.move_to_end(key)
            return h
    nufft_type, dim, single, nk, iflag, ntr, eps, nopts, stream = key[:9]
    native = to_native_from_key(nopts)
    plan = ctypes.c_void_p()
    nm = (ctypes.c_int64 * 3)(*nk)
    mk = lib.gbnf_makeplan if single else lib.gbn_makeplan
    _native.check(mk(nufft_type, dim, nm, iflag, ntr, eps, ctypes.byref(plan),
                     ctypes.byref(native), ctypes.c_void_p(stream or None)), "makeplan")
    entry = (plan, threading.Lock())
    evict = []
    with _lock:
        if key in _plans:  # another thread made it meanwhile
            lib.gbn_destroy(plan)
            return _plans[key]
        _plans[key] = entry
        while len(_plans) > _MAX_PLANS:
            evict.append(_plans.popitem(last=False)[1])
    for p, plock in evict:
        with plock:  # wait for a call in flight on it
            lib.gbn_destroy(p)
    return entry


def to_native_from_key(nopts):
    n = _native.GbnOpts()
    for (f, _), v in zip(n._fields_, nopts):
        setattr(n, f, v)
    return n


class FusedState:
    """A forward's plan key and its point sets (one per n_tot index)."""

    def __init__(self, key, handles):
        self.key = key
        self.handles = handles

    def __del__(self):
        try:
            lib = _native.load()
            for h in self.handles:
                lib.gbn_points_destroy(h)
        except Exception:  # interpreter shutdown
            pass
        self.handles = []


def plan_key(nufft_type, dim, single, nk_b, iflag, n_transf, eps_v, opts, device, stream,
             n_j=0):
    fwd = unpack_opts(opts, nufft_type, True) or Opts()
    native = to_native(fwd)
    if getattr(fwd, "gpu_autotune", False) and n_j > 0:
        from . import tune

        native, _ = tune.tuned_native(nufft_type, dim, single, nk_b, n_j, n_transf, eps_v,
                                      iflag, native, stream)
    return (nufft_type, dim, bool(single), tuple(int(v) for v in nk_b), int(iflag), int(n_transf),
            float(eps_v), _opts_key(native), int(stream), str(device))


def forward(nufft_type, source, points, output_shape, iflag, eps, opts, out, single, dim):
    """Run a type-1/2 forward keeping its point sets; returns a FusedState."""
    lib = _native.load()
    dev = source.device
    n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
    n_j = int(points[0].shape[1])
    if nufft_type == 1:
        nk = tuple(int(n) for n in output_shape)
    else:
        nk = tuple(int(n) for n in source.shape[2:])
    nk_b = list(nk[::-1]) + [1] * (3 - dim)
    eps_v = float(np.float32(eps)) if single else float(eps)
    stream = torch.cuda.current_stream(dev).cuda_stream
    key = plan_key(nufft_type, dim, single, nk_b, iflag, n_transf, eps_v, opts, dev, stream,
                   n_j)
    plan, plock = get_plan(key)
    src = source.contiguous()
    pts = [p.contiguous() for p in points][::-1]  # backend order
    esz = src.element_size()
    psz = pts[0].element_size()
    n_k_total = int(np.prod(nk))
    handles = []
    try:
        plock.acquire()
        for idx in range(n_tot):
            h = ctypes.c_void_p()
            xs = [ctypes.c_void_p(p.data_ptr() + idx * n_j * psz) for p in pts] + [None] * (3 - dim)
            _native.check(lib.gbn_points_create(plan, n_j, xs[0], xs[1], xs[2], ctypes.byref(h)),
                          "setpts")
            handles.append(h)
            c_off = idx * n_j * n_transf * esz
            f_off = idx * n_k_total * n_transf * esz
            if nufft_type == 1:
                c_ptr, f_ptr = src.data_ptr() + c_off, out.data_ptr() + f_off
            else:
                c_ptr, f_ptr = out.data_ptr() + c_off, src.data_ptr() + f_off
            _native.check(lib.gbn_execute_points(plan, h, n_transf, 1, ctypes.c_void_p(c_ptr),
                                                 ctypes.c_void_p(f_ptr)), "execute")
    except Exception:
        for h in handles:
            lib.gbn_points_destroy(h)
        raise
    finally:
        plock.release()
    return FusedState(key, handles)


def backward(state, nufft_type, source, points, g, need_src, need_pts):
    """Fused gradients: (grad_source or None, [grad per point array or None])."""
    lib = _native.load()
    plan, plock = get_plan(state.key)
    dim = len(points)
    n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
    n_j = int(points[0].shape[1])
    src = source.contiguous()
    g = g.contiguous()
    esz = src.element_size()
    grad_src = torch.empty_like(src) if need_src else None
    grads = [torch.empty(points[u].shape, dtype=points[u].dtype, device=src.device)
             if need_pts[u] else None for u in range(dim)]
    psz = points[0].element_size()
    per_src = src[0].numel() * esz  # bytes per n_tot index of the source
    per_g = g[0].numel() * esz
    with plock:
        _backward_calls(lib, plan, state, n_tot, n_transf, n_j, dim, src, g, grad_src, grads,
                        psz, per_src, per_g)
    return grad_src, grads


def _backward_calls(lib, plan, state, n_tot, n_transf, n_j, dim, src, g, grad_src, grads, psz,
                    per_src, per_g):
    for idx in range(n_tot):
        gx = (ctypes.c_void_p * 3)()
        for u in range(dim):
            d = dim - 1 - u  # backend axis of user axis u
            if grads[u] is not None:
                gx[d] = grads[u].data_ptr() + idx * n_j * psz
        gs = grad_src.data_ptr() + idx * per_src if grad_src is not None else None
        _native.check(lib.gbn_grad(plan, state.handles[idx], n_transf,
                                   ctypes.c_void_p(src.data_ptr() + idx * per_src),
                                   ctypes.c_void_p(g.data_ptr() + idx * per_g),
                                   ctypes.c_void_p(gs) if gs else None, gx), "grad")


# -- type 3 ------------------------------------------------------------------------
# A type-3 plan holds its point sets (sources sorted for the spreading grid,
# rescaled targets sorted for the inner type 2) and its phase factors, so a
# differentiable forward keeps whole plans (one per n_tot index) for the
# backward.  Idle plans are pooled per key; setpts reuses a plan's inner
# type-2 plan while the grid size stays the same.
_t3_pool = {}
_T3_POOL_MAX = 4


def _t3_take(key):
    with _lock:
        idle = _t3_pool.get(key)
        if idle:
            return idle.pop()
    lib = _native.load()
    dim, single, iflag, ntr, eps, nopts, stream = key[:7]
    native = to_native_from_key(nopts)
    plan = ctypes.c_void_p()
    mk = lib.gbnf_makeplan if single else lib.gbn_makeplan
    _native.check(mk(3, dim, None, iflag, ntr, eps, ctypes.byref(plan), ctypes.byref(native),
                     ctypes.c_void_p(stream or None)), "makeplan")
    return plan


def _t3_give(key, plans):
    lib = _native.load()
    extra = []
    with _lock:
        idle = _t3_pool.setdefault(key, [])
        for p in plans:
            (idle if len(idle) < _T3_POOL_MAX else extra).append(p)
    for p in extra:
        lib.gbn_destroy(p)


class T3State:
    """A type-3 forward's plans (one per n_tot index), returned to the pool
    when the state goes away."""

    def __init__(self, key, plans):
        self.key = key
        self.plans = plans

    def __del__(self):
        try:
            _t3_give(self.key, self.plans)
        except Exception:  # interpreter shutdown
            pass
        self.plans = []


def t3_forward(source, points, iflag, eps, opts, out, single, dim):
    """Type-3 forward keeping its plans; returns a T3State."""
    lib = _native.load()
    dev = source.device
    n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
    n_j = int(points[0].shape[1])
    n_k = int(points[dim].shape[1])
    eps_v = float(np.float32(eps)) if single else float(eps)
    stream = torch.cuda.current_stream(dev).cuda_stream
    native = to_native(unpack_opts(opts, 3, True) or Opts())
    key = (dim, bool(single), int(iflag), n_transf, eps_v, _opts_key(native), int(stream),
           str(dev))
    src = source.contiguous()
    xs = [p.contiguous() for p in points[:dim]][::-1]  # backend order
    ss = [p.contiguous() for p in points[dim:]][::-1]
    esz = src.element_size()
    psz = xs[0].element_size()
    setpts = lib.gbnf_setpts if single else lib.gbn_setpts
    plans = []
    try:
        for idx in range(n_tot):
            plan = _t3_take(key)
            plans.append(plan)
            xp = [ctypes.c_void_p(p.data_ptr() + idx * n_j * psz) for p in xs] + [None] * (3 - dim)
            sp = [ctypes.c_void_p(p.data_ptr() + idx * n_k * psz) for p in ss] + [None] * (3 - dim)
            _native.check(setpts(plan, n_j, *xp, n_k, *sp), "setpts")
            _native.check(lib.gbn_execute(
                plan, ctypes.c_void_p(src.data_ptr() + idx * n_j * n_transf * esz),
                ctypes.c_void_p(out.data_ptr() + idx * n_k * n_transf * esz)), "execute")
    except Exception:
        _t3_give(key, plans)
        raise
    return T3State(key, plans)


def t3_backward(state, source, points, g, need_src, need_pts):
    """Fused type-3 gradients for the strengths and the source points (one
    adjoint pass per n_tot index whose gather also differentiates along the
    sources); target gradients are not part of it."""
    lib = _native.load()
    dim = len(points) // 2
    n_tot, n_transf = int(source.shape[0]), int(source.shape[1])
    n_j = int(points[0].shape[1])
    src = source.contiguous()
    g = g.contiguous()
    esz = src.element_size()
    grad_src = torch.empty_like(src) if need_src else None
    grads = [torch.empty(points[u].shape, dtype=points[u].dtype, device=src.device)
             if need_pts[u] else None for u in range(dim)]
    psz = points[0].element_size()
    per_src = src[0].numel() * esz
    per_g = g[0].numel() * esz
    for idx in range(n_tot):
        gx = (ctypes.c_void_p * 3)()
        for u in range(dim):
            if grads[u] is not None:
                gx[dim - 1 - u] = grads[u].data_ptr() + idx * n_j * psz
        gs = grad_src.data_ptr() + idx * per_src if grad_src is not None else None
        _native.check(lib.gbn_grad(state.plans[idx], None, n_transf,
                                   ctypes.c_void_p(src.data_ptr() + idx * per_src),
                                   ctypes.c_void_p(g.data_ptr() + idx * per_g),
                                   ctypes.c_void_p(gs) if gs else None, gx), "grad")
    return grad_src, grads
