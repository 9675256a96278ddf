"""Autotuned execution settings for type-1/2 transforms (``gbn_autotune``).

The reference fixes sigma, method, bin sizes and subproblem size per call
through its options (src/jax_finufft/options.py:46-119).  Here the library
can time candidates on synthetic points of the same class (type, dimension,
precision, mode shape, point count rounded up to a power of two, transforms
per call, tolerance) and keep the fastest one that stays as accurate as the
default settings; the choice is cached in memory and on disk.

``autotune`` returns an ``Opts`` carrying the chosen settings, to pass to
nufft1/nufft2 or NufftBatch.  ``Opts(gpu_autotune=True)`` makes nufft1 and
nufft2 look the settings up (tuning on a cache miss) on every call.
"""
import ctypes
import dataclasses

import numpy as np
import torch

from . import _native
from .options import Opts, to_native, unpack_opts

__all__ = ["autotune", "clear_cache"]

TUNE_ON, TUNE_SM_ONLY, TUNE_KEEP_SIGMA = 1, 2, 4


def tuned_native(nufft_type, dim, single, nk_b, M, n_transf, eps, iflag, native, stream,
                 flags=TUNE_ON):
    """GbnOpts with the tuned settings of one class (the library's cache or a
    tuning run on `stream`); returns (opts, info dict)."""
    lib = _native.load()
    base = _native.GbnOpts()
    ctypes.pointer(base)[0] = native
    base.gpu_autotune = int(flags)
    out = _native.GbnOpts()
    info = (ctypes.c_double * 3)()
    nm = (ctypes.c_int64 * 3)(*[int(v) for v in nk_b])
    _native.check(lib.gbn_autotune(int(nufft_type), int(dim), int(bool(single)), nm, int(M),
                                   int(n_transf), float(eps), int(iflag), ctypes.byref(base),
                                   ctypes.c_void_p(int(stream) or None), ctypes.byref(out), info),
                  "autotune")
    return out, {"ms": info[0], "rel_err": info[1], "cached": bool(info[2])}


def autotune(nufft_type, n_modes, n_points, ntransf=1, eps=1e-6, dtype=torch.complex64,
             opts=None, iflag=None, device=None, keep_sigma=False):
    """Tune one class and return (Opts with the chosen settings, info).

    n_modes: mode shape in the user's axis order; n_points: M.  info holds
    the median time of one setpts + execute on the synthetic problem, its
    relative error against an FP64 transform, and whether it came from the
    cache."""
    if nufft_type not in (1, 2):
        raise ValueError("autotune supports types 1 and 2")
    n_modes = tuple(int(n) for n in n_modes)
    dim = len(n_modes)
    single = dtype == torch.complex64
    fwd = unpack_opts(opts, nufft_type, True) or Opts()
    if iflag is None:
        iflag = 1 if nufft_type == 1 else -1
    eps_v = float(np.float32(eps)) if single else float(eps)
    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    nk_b = list(n_modes[::-1]) + [1] * (3 - dim)
    flags = TUNE_ON | (TUNE_KEEP_SIGMA if keep_sigma else 0)
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev).cuda_stream
        nat, info = tuned_native(nufft_type, dim, single, nk_b, n_points, ntransf, eps_v, iflag,
                                 to_native(fwd), stream, flags)
    tuned = dataclasses.replace(
        fwd, gpu_upsampfac=float(nat.upsampfac), gpu_method=int(nat.gpu_method),
        gpu_binsizex=int(nat.gpu_binsizex), gpu_binsizey=int(nat.gpu_binsizey),
        gpu_binsizez=int(nat.gpu_binsizez), gpu_maxsubprobsize=int(nat.gpu_maxsubprobsize),
        gpu_autotune=False)
    return tuned, info


def clear_cache(forget_file=False):
    """Forget the in-memory tuning results (and, with forget_file, do not
    reload the cache file in this process)."""
    _native.load().gbn_autotune_clear(int(bool(forget_file)))
