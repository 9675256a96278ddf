"""Batched plans: many independent type-1/2 problems in one pass.

The reference runs independent point sets of one shape through a host loop
(lib/kernels.cc.cu:57-80) and problems of different shapes as separate FFI
calls.  ``NufftBatch`` hands K problems -- each with its own points, point
count and mode shape, all sharing type, dimension, precision, sign and
tolerance -- to ``gbn_batch_run``: per-problem sorting and deconvolution,
one batched cuFFT per group of equal grid shapes, and one persistent
spread/interpolation kernel over a (problem, subproblem, transform) work
queue, optionally captured as a CUDA graph and replayed.

Axes are in the user's order (as nufft1/nufft2); packing is problem after
problem (see include/gbnufft.h, gbn_batch_create).
"""
import ctypes

import numpy as np
import torch

from . import _native
from .options import Opts, to_native

__all__ = ["NufftBatch", "NufftBatchChain"]


class NufftBatch:
    """K independent NUFFTs of one type executed together.

    nufft_type: 1 (points -> modes) or 2 (modes -> points).
    n_modes: K mode shapes (user axis order, same dimension for all).
    n_points: K point counts.
    ntransf: transforms per problem (stacked strengths/modes).
    upsampfac: optional K upsampling factors (sigma per problem).
    autotune: pick each problem's sigma (unless upsampfac is given), bin size
        and points per subproblem with the autotuner (cached per class).

    Work runs on a stream the batch owns (the legacy default stream cannot be
    captured into a graph), ordered after everything already queued on the
    stream that was current at construction and before anything queued on it
    afterwards.
    """

    def __init__(self, nufft_type, n_modes, n_points, ntransf=1, iflag=None, eps=1e-6,
                 dtype=torch.complex64, opts=None, upsampfac=None, device=None,
                 use_graph=True, autotune=False):
        if nufft_type not in (1, 2):
            raise ValueError("NufftBatch supports types 1 and 2")
        self.type = nufft_type
        self.shapes = [tuple(int(n) for n in s) for s in n_modes]
        self.dim = len(self.shapes[0])
        if any(len(s) != self.dim for s in self.shapes):
            raise ValueError("all problems must have the same dimension")
        self.M = [int(m) for m in n_points]
        if len(self.M) != len(self.shapes):
            raise ValueError("n_modes and n_points must have the same length")
        self.K = len(self.M)
        self.T = int(ntransf)
        self.iflag = (1 if nufft_type == 1 else -1) if iflag is None else int(iflag)
        self.dtype = dtype
        self.single = dtype == torch.complex64
        self.rdtype = torch.float32 if self.single else torch.float64
        self.device = torch.device(device or "cuda", torch.cuda.current_device()) \
            if device is None else torch.device(device)
        self.use_graph = use_graph
        self.lib = _native.load()
        nm = (ctypes.c_int64 * (3 * self.K))()
        for k, s in enumerate(self.shapes):
            b = list(s[::-1]) + [1] * (3 - self.dim)
            for d in range(3):
                nm[3 * k + d] = b[d]
        Ms = (ctypes.c_int64 * self.K)(*self.M)
        sig = None
        if upsampfac is not None:
            sig = (ctypes.c_double * self.K)(*[float(v) for v in upsampfac])
        native = to_native(opts or Opts())
        if autotune:
            native.gpu_autotune = 1  # per problem, shared-memory method (work queue)
        eps_v = float(np.float32(eps)) if self.single else float(eps)
        self.stream = torch.cuda.current_stream(self.device)
        self.handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self.lib.gbn_batch_create(
                nufft_type, self.dim, int(self.single), self.K, nm, Ms, sig, self.T, self.iflag,
                eps_v, ctypes.byref(native), ctypes.c_void_p(self.stream.cuda_stream),
                ctypes.byref(self.handle)), "batch_create")
        self.pt_off = np.concatenate([[0], np.cumsum(self.M)]).astype(np.int64)
        self.mode_sizes = [int(np.prod(s)) for s in self.shapes]
        self.mode_off = np.concatenate([[0], np.cumsum(self.mode_sizes)]).astype(np.int64)

    def __del__(self):
        try:
            if self.handle:
                self.lib.gbn_batch_destroy(self.handle)
        except Exception:
            pass
        self.handle = None

    def info(self):
        ng, q, ab = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        _native.check(self.lib.gbn_batch_info(self.handle, ctypes.byref(ng), ctypes.byref(q),
                                              ctypes.byref(ab)))
        return {"fft_groups": ng.value, "work_queue": bool(q.value), "arena_bytes": ab.value}

    # -- packed interface ------------------------------------------------------
    def empty_points(self):
        """Packed point arrays (dim x sum M), user axis order."""
        return torch.empty((self.dim, int(self.pt_off[-1])), dtype=self.rdtype,
                           device=self.device)

    def empty_strengths(self):
        return torch.empty(self.T * int(self.pt_off[-1]), dtype=self.dtype, device=self.device)

    def empty_modes(self):
        return torch.empty(self.T * int(self.mode_off[-1]), dtype=self.dtype, device=self.device)

    def run_packed(self, points, c, f):
        """One pass on packed buffers (points: (dim, sum M) user order; type 1:
        c -> f, type 2: f -> c).  Buffers must stay at the same addresses for
        the captured graph to be replayed."""
        pts = [points[u] for u in range(self.dim)][::-1]  # backend order
        ptr = [ctypes.c_void_p(p.data_ptr()) for p in pts] + [None] * (3 - self.dim)
        with torch.cuda.device(self.device):
            _native.check(self.lib.gbn_batch_run(self.handle, ptr[0], ptr[1], ptr[2],
                                                 ctypes.c_void_p(c.data_ptr()),
                                                 ctypes.c_void_p(f.data_ptr()),
                                                 int(self.use_graph)), "batch_run")

    # -- list interface ------------------------------------------------------------
    def pack_points(self, points):
        """points: K tuples of dim arrays of M_k points each (user order)."""
        out = self.empty_points()
        for k, pk in enumerate(points):
            for u in range(self.dim):
                out[u, self.pt_off[k]:self.pt_off[k + 1]] = torch.as_tensor(pk[u])
        return out

    def __call__(self, points, sources):
        """Type 1: sources = K strength arrays (T, M_k) or (M_k,) -> K mode arrays.
        Type 2: sources = K mode arrays (T, *N_k) or N_k -> K value arrays."""
        P = self.pack_points(points)
        if self.type == 1:
            c = torch.cat([torch.as_tensor(s, device=self.device).to(self.dtype)
                           .reshape(self.T, -1).reshape(-1) for s in sources])
            f = self.empty_modes()
            self.run_packed(P, c, f)
            outs = []
            for k, s in enumerate(self.shapes):
                o = f[self.T * self.mode_off[k]:self.T * self.mode_off[k + 1]]
                outs.append(o.reshape((self.T,) + s) if self.T > 1 else o.reshape(s))
            return outs
        f = torch.cat([torch.as_tensor(s, device=self.device).to(self.dtype).reshape(-1)
                       for s in sources])
        c = self.empty_strengths()
        self.run_packed(P, c, f)
        outs = []
        for k in range(self.K):
            o = c[self.T * self.pt_off[k]:self.T * self.pt_off[k + 1]]
            outs.append(o.reshape(self.T, -1) if self.T > 1 else o)
        return outs


class NufftBatchChain:
    """Several NufftBatch objects (of either type) run as one pass.

    Each batch runs on its own stream, forked from and joined back to the
    chain's stream so the batches overlap, and the whole pass is captured
    into one CUDA graph on the first call and replayed while the buffers
    stay at the same addresses (gbn_batch_chain_run).  The chain keeps its
    batches alive; do not run them on their own while the chain is in use.
    """

    def __init__(self, batches, use_graph=True):
        self.batches = list(batches)
        if not self.batches:
            raise ValueError("a chain needs at least one batch")
        self.lib = _native.load()
        self.use_graph = use_graph
        dev = self.batches[0].device
        if any(b.device != dev for b in self.batches):
            raise ValueError("all batches of a chain must be on one device")
        self.device = dev
        self.stream = torch.cuda.current_stream(dev)
        arr = (ctypes.c_void_p * len(self.batches))(*[b.handle.value for b in self.batches])
        self.handle = ctypes.c_void_p()
        with torch.cuda.device(dev):
            _native.check(self.lib.gbn_batch_chain_create(
                arr, len(self.batches), ctypes.c_void_p(self.stream.cuda_stream),
                ctypes.byref(self.handle)), "batch_chain_create")

    def __del__(self):
        try:
            if self.handle:
                self.lib.gbn_batch_chain_destroy(self.handle)
        except Exception:
            pass
        self.handle = None

    def run_packed(self, args):
        """args: one (points, c, f) tuple per batch, as NufftBatch.run_packed."""
        n = len(self.batches)
        if len(args) != n:
            raise ValueError("one (points, c, f) tuple per batch")
        X, Y, Z, C, F = [(ctypes.c_void_p * n)() for _ in range(5)]
        for i, (b, (points, c, f)) in enumerate(zip(self.batches, args)):
            pts = [points[u] for u in range(b.dim)][::-1]  # backend order
            ptr = [p.data_ptr() for p in pts] + [None] * (3 - b.dim)
            X[i], Y[i], Z[i] = ptr
            C[i], F[i] = c.data_ptr(), f.data_ptr()
        with torch.cuda.device(self.device):
            _native.check(self.lib.gbn_batch_chain_run(self.handle, X, Y, Z, C, F,
                                                       int(self.use_graph)), "batch_chain_run")
