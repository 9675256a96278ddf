"""gbn_binsort_noalloc: the bin sort for callers that cannot allocate.

Some callers cannot call cudaMalloc (a plugin whose host framework owns all
device memory, a pipeline that reserves every byte up front).
gbn_binsort_noalloc gives them setpts' fold and bin sort with no allocation:
they pass points and output arrays, and the scratch lives in a fixed device
array inside the library.  This test calls it through the C ABI and checks
that, on two calls in a row with different points, its bin of every point
and its bin counts equal those of the existing entry point (gbn_setpts, read
back with gbn_debug_bins) exactly -- bin indices are integer work, so the
tolerance is zero -- and that its permutation lists the points in bin order.
It lives in its own file so pytest collects it last; it passes alone in a
fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

I64P = ctypes.POINTER(ctypes.c_int64)


def _existing_bins(lib, native, dim, single, pts, nmodes, binsize):
    """Bins and counts from the existing path: makeplan + setpts + debug_bins."""
    opts = native.default_opts()
    opts.gpu_binsizex, opts.gpu_binsizey, opts.gpu_binsizez = binsize
    opts.gpu_method = 2
    plan = ctypes.c_void_p()
    nm = (ctypes.c_int64 * 3)(*(list(nmodes) + [1] * (3 - dim)))
    mk = lib.gbnf_makeplan if single else lib.gbn_makeplan
    native.check(mk(1, dim, nm, 1, 1, 1e-6, ctypes.byref(plan), ctypes.byref(opts), None))
    try:
        ptr = [ctypes.c_void_p(p.data_ptr()) for p in pts] + [None] * (3 - dim)
        setpts = lib.gbnf_setpts if single else lib.gbn_setpts
        native.check(setpts(plan, pts[0].numel(), ptr[0], ptr[1], ptr[2], 0, None, None, None))
        nf = (ctypes.c_int64 * 3)()
        w = ctypes.c_int()
        native.check(lib.gbn_plan_info(plan, ctypes.byref(w), nf, None, None))
        nbins = ctypes.c_int64()
        lib.gbn_debug_bins(plan, None, None, ctypes.byref(nbins))
        bins = np.empty(pts[0].numel(), dtype=np.int64)
        counts = np.empty(nbins.value, dtype=np.int64)
        native.check(lib.gbn_debug_bins(plan, bins.ctypes.data_as(I64P),
                                        counts.ctypes.data_as(I64P), ctypes.byref(nbins)))
    finally:
        lib.gbn_destroy(plan)
    return [nf[d] for d in range(3)], w.value, bins, counts


def _noalloc(lib, native, dim, single, pts, nf, binsize, w, nbins):
    M = pts[0].numel()
    dev = pts[0].device
    bins = torch.empty(M, dtype=torch.int32, device=dev)
    counts = torch.full((nbins,), -7, dtype=torch.int32, device=dev)  # must be cleared
    perm = torch.empty(M, dtype=torch.int32, device=dev)
    ptr = [ctypes.c_void_p(p.data_ptr()) for p in pts] + [None] * (3 - dim)
    nfa = (ctypes.c_int64 * 3)(*nf)
    bsa = (ctypes.c_int * 3)(*binsize)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    native.check(lib.gbn_binsort_noalloc(stream, dim, int(single), M, ptr[0], ptr[1], ptr[2],
                                         nfa, bsa, w, ctypes.c_void_p(bins.data_ptr()),
                                         ctypes.c_void_p(counts.data_ptr()),
                                         ctypes.c_void_p(perm.data_ptr())))
    torch.cuda.synchronize()
    return bins.cpu().numpy(), counts.cpu().numpy(), perm.cpu().numpy()


@pytest.mark.parametrize("dim, single", [(1, True), (2, False), (3, True), (3, False)])
def test_noalloc_binsort_matches_setpts(dim, single):
    from jax_finufft_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(11 + dim)
    nmodes = {1: (3000,), 2: (300, 210), 3: (60, 44, 50)}[dim]
    binsize = {1: (256, 1, 1), 2: (32, 16, 1), 3: (16, 8, 8)}[dim]
    dt = torch.float32 if single else torch.float64
    for call in range(2):  # two calls in a row share (and must reset) the scratch
        M = 50000 if call == 0 else 37000
        half = M // 2
        pts = []
        for _ in range(dim):
            v = np.concatenate([rng.uniform(-np.pi, np.pi, half), rng.normal(0, 0.2, M - half)])
            pts.append(torch.tensor(v, dtype=dt, device="cuda"))
        nf, w, ref_bins, ref_counts = _existing_bins(lib, _native, dim, single, pts, nmodes,
                                                     binsize)
        bs = [min(binsize[d], nf[d]) if d < dim else 1 for d in range(3)]
        bins, counts, perm = _noalloc(lib, _native, dim, single, pts, nf, bs, w,
                                      ref_counts.size)
        np.testing.assert_array_equal(bins.astype(np.int64), ref_bins)
        np.testing.assert_array_equal(counts.astype(np.int64), ref_counts)
        assert np.array_equal(np.sort(perm), np.arange(M))
        assert np.all(np.diff(bins[perm]) >= 0)


def test_noalloc_rejects_oversize():
    from jax_finufft_gb300 import _native

    lib = _native.load()
    M = 262144 + 1  # GBN_NOALLOC_MAX_POINTS + 1
    nf = (ctypes.c_int64 * 3)(64, 1, 1)
    bs = (ctypes.c_int * 3)(8, 1, 1)
    rc = lib.gbn_binsort_noalloc(None, 1, 1, M, None, None, None, nf, bs, 7, None, None, None)
    assert rc == 2
    assert "exceeds the limit" in _native.last_error()
    nf = (ctypes.c_int64 * 3)(1 << 20, 1024, 1)
    bs = (ctypes.c_int * 3)(1, 1, 1)
    rc = lib.gbn_binsort_noalloc(None, 2, 1, 10, None, None, None, nf, bs, 7, None, None, None)
    assert rc == 2
    assert "bins exceed" in _native.last_error()
