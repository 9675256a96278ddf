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


def _edge_coords(rng, M):
    """Uniform draws with the fold's edge values planted at the front: the
    period ends +-pi, 0, +-2pi, values many periods out, the float32 neighbours
    of pi, and non-finite entries (which fold as 0)."""
    v = rng.uniform(-np.pi, np.pi, M)
    f32pi = float(np.float32(np.pi))
    edges = [np.pi, -np.pi, 0.0, -0.0, 2 * np.pi, -2 * np.pi, 1e6, -1e6, f32pi,
             float(np.nextafter(np.float32(np.pi), np.float32(0))),
             float(np.nextafter(np.float32(-np.pi), np.float32(0))),
             np.nan, np.inf, -np.inf]
    v[: len(edges)] = edges
    return v


@pytest.mark.parametrize("single", [True, False])
def test_noalloc_at_limits_matches_oracle(single):
    """M = GBN_NOALLOC_MAX_POINTS points into GBN_NOALLOC_MAX_BINS bins (a
    512 x 512 fine grid in 1 x 1 bins), with edge and non-finite coordinates:
    every bin equals the oracle fold's bin (oracle/nufft_oracle.c
    orc_fold_points; the FP32 coordinates are exact in FP64, and the library
    folds both precisions on the FP64 chain), counts are the bins' histogram,
    and perm is a permutation in bin order."""
    from jax_finufft_gb300 import _native
    from oracle import cpu_nufft as cn

    lib = _native.load()
    rng = np.random.default_rng(23)
    M, nf, bs, w = 262144, [512, 512, 1], [1, 1, 1], 7
    dt = torch.float32 if single else torch.float64
    npdt = np.float32 if single else np.float64
    coords = [_edge_coords(rng, M).astype(npdt), _edge_coords(rng, M)[::-1].astype(npdt)]
    pts = [torch.tensor(np.ascontiguousarray(v), device="cuda") for v in coords]
    assert pts[0].dtype == dt
    bins, counts, perm = _noalloc(lib, _native, 2, single, pts, nf, bs, w, 512 * 512)
    _, _, _, ref_bins = cn.fold_points([v.astype(np.float64) for v in coords], nf[:2], w, bs[:2])
    np.testing.assert_array_equal(bins.astype(np.int64), ref_bins)
    np.testing.assert_array_equal(counts, np.bincount(ref_bins, minlength=512 * 512))
    assert np.array_equal(np.sort(perm), np.arange(M))
    assert np.all(np.diff(bins[perm]) >= 0)


def test_noalloc_no_points_clears_counts():
    """M = 0: the point and per-point output arrays may be NULL; counts is
    still written (all zeros)."""
    from jax_finufft_gb300 import _native

    lib = _native.load()
    counts = torch.full((64 * 8,), -7, dtype=torch.int32, device="cuda")
    nf = (ctypes.c_int64 * 3)(64, 64, 1)
    bs = (ctypes.c_int * 3)(8, 1, 1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _native.check(lib.gbn_binsort_noalloc(stream, 2, 0, 0, None, None, None, nf, bs, 5, None,
                                          ctypes.c_void_p(counts.data_ptr()), None))
    torch.cuda.synchronize()
    assert torch.count_nonzero(counts).item() == 0
