"""Host-side logic on CPU: shape flattening, options, and the C ABI surface."""
import ctypes
import os
import re

import pytest
import torch

from jax_finufft_gb300 import options, shapes


# --- shapes (port of the reference's tests/shapes_test.py) ------------------
def test_broadcast_inputs():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        1, (10,), torch.empty((50, 5, 1, 7, 12, 5)), torch.empty((50, 1, 6, 1, 12, 5)))
    assert source.shape == (50 * 6 * 12, 5 * 7, 5)
    assert len(points) == 1
    assert points[0].shape == (50 * 6 * 12, 5)
    assert index.broadcast_from == (1, 3)
    assert index.broadcast_to == (3, 4)
    assert index.expected_output_shape == (50, 6, 12, 5, 7, 10)


def test_broadcast_inputs_type2():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        2, None, torch.empty((50, 5, 1, 7, 12, 11)), torch.empty((50, 1, 6, 1, 12, 5)))
    assert source.shape == (50 * 6 * 12, 5 * 7, 11)
    assert points[0].shape == (50 * 6 * 12, 5)
    assert index.broadcast_from == (1, 3)
    assert index.broadcast_to == (3, 4)
    assert index.expected_output_shape == (50, 6, 12, 5, 7, 5)


def test_vector_inputs():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        2, None, torch.empty((5, 6)), torch.empty((10,)), torch.empty((10,)))
    assert source.shape == (1, 1, 5, 6)
    assert [p.shape for p in points] == [(1, 10), (1, 10)]
    assert index.expected_output_shape == (10,)
    assert index.broadcast_from == () and index.broadcast_to == ()


def test_unpadded_points_type2():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        2, None, torch.empty((3, 8, 5, 6)), torch.empty((3, 10)), torch.empty((3, 10)))
    assert source.shape == (3, 8, 5, 6)
    assert [p.shape for p in points] == [(3, 10), (3, 10)]
    assert index.expected_output_shape == (3, 8, 10)
    assert index.broadcast_from == (1,) and index.broadcast_to == (1,)


def test_unpadded_points_type1():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        1, (17, 13), torch.empty((3, 5, 6)), torch.empty((1, 6)), torch.empty((1, 6)))
    assert source.shape == (1, 3 * 5, 6)
    assert [p.shape for p in points] == [(1, 6), (1, 6)]
    assert index.expected_output_shape == (3, 5, 17, 13)
    assert index.broadcast_from == (0, 1) and index.broadcast_to == (0, 1)


def test_unpadded_points_type3():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        3, None, torch.empty((3, 5, 6)), torch.empty((3, 6)), torch.empty((3, 6)),
        torch.empty((3, 11)), torch.empty((3, 11)))
    assert source.shape == (3, 5, 6)
    assert [p.shape for p in points] == [(3, 6), (3, 6), (3, 11), (3, 11)]
    assert index.expected_output_shape == (3, 5, 11)
    assert index.broadcast_from == (1,) and index.broadcast_to == (1,)


def test_type3():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        3, None, torch.empty((13, 3, 5, 7, 11)), torch.empty((13, 1, 5, 1, 11)),
        torch.empty((1, 5, 1, 23)))
    assert source.shape == (13 * 5, 3 * 7, 11)
    assert [p.shape for p in points] == [(13 * 5, 11), (13 * 5, 23)]
    assert index.expected_output_shape == (13, 5, 3, 7, 23)
    assert index.broadcast_from == (1, 3) and index.broadcast_to == (2, 3)


def test_type3_2d():
    index, source, *points = shapes.broadcast_and_flatten_inputs(
        3, None, torch.empty((13, 3, 5, 7, 11)), torch.empty((13, 1, 5, 1, 11)),
        torch.empty((1, 5, 1, 11)), torch.empty((5, 1, 23)), torch.empty((1, 23)))
    assert source.shape == (13 * 5, 3 * 7, 11)
    assert [p.shape for p in points] == [(65, 11), (65, 11), (65, 23), (65, 23)]
    assert index.expected_output_shape == (13, 5, 3, 7, 23)
    assert index.broadcast_from == (1, 3) and index.broadcast_to == (2, 3)


def test_unflatten_roundtrip():
    idx, source, *pts = shapes.broadcast_and_flatten_inputs(
        1, (4,), torch.arange(2 * 3 * 5, dtype=torch.float64).reshape(2, 3, 5),
        torch.zeros(2, 1, 5))
    res = torch.arange(source.shape[0] * source.shape[1] * 4, dtype=torch.float64).reshape(
        source.shape[0], source.shape[1], 4)
    out = idx.unflatten(res)
    assert tuple(out.shape) == (2, 3, 4)


def _general_path(monkeypatch, *args):
    monkeypatch.setattr(shapes, "_flat_vector_points", lambda *a: None)
    try:
        return shapes.broadcast_and_flatten_inputs(*args)
    finally:
        monkeypatch.undo()


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("M", [1, 7])
@pytest.mark.parametrize("T", [None, 1, 3])
def test_vector_points_fast_path_matches_general_rules(monkeypatch, dim, M, T):
    """One set of 1-D points (the common call): the shortcut's buffers, output
    shape and unflattening equal the general broadcasting rules' for types
    1, 2 and 3."""
    g = torch.Generator().manual_seed(dim * 100 + M)
    pts = [torch.randn(M, generator=g) for _ in range(dim)]
    modes = (4, 5, 6)[:dim]
    src1 = torch.randn(M, generator=g) if T is None else torch.randn(T, M, generator=g)
    src2 = torch.randn(*modes, generator=g) if T is None else torch.randn(T, *modes, generator=g)
    tgts = [torch.randn(5, generator=g) for _ in range(dim)]
    cases = [(1, modes, src1, pts), (2, None, src2, pts), (3, None, src1, pts + tgts)]
    for t, out_shape, src, ps in cases:
        fast = shapes.broadcast_and_flatten_inputs(t, out_shape, src, *ps)
        ref = _general_path(monkeypatch, t, out_shape, src, *ps)
        assert tuple(fast[0].expected_output_shape) == tuple(ref[0].expected_output_shape)
        for a, b in zip(fast[1:], ref[1:]):
            assert a.shape == b.shape and torch.equal(a, b)
        n_out = {1: modes, 2: (M,), 3: (5,)}[t]
        res = torch.randn(*fast[1].shape[:2], *n_out, generator=g)
        assert torch.equal(fast[0].unflatten(res), ref[0].unflatten(res))


def test_vector_points_of_different_lengths_take_the_general_path():
    with pytest.raises((AssertionError, RuntimeError)):
        shapes.broadcast_and_flatten_inputs(1, (4, 4), torch.zeros(5), torch.zeros(5),
                                            torch.zeros(6))


# --- options (port of the reference's tests/options_test.py) ------------------
@pytest.mark.parametrize("opts", [None, options.Opts()])
def test_default_options(opts):
    for t in (1, 2):
        for fwd in (True, False):
            assert options.unpack_opts(opts, t, fwd) == opts


def test_nested_by_type():
    opts = options.NestedOpts(type1=options.Opts(spread_debug=True),
                              type2=options.Opts(debug=True))
    assert options.unpack_opts(opts, 1, True) == options.Opts(spread_debug=True)
    assert options.unpack_opts(opts, 2, True) == options.Opts(debug=True)


def test_nested_by_direction():
    opts = options.NestedOpts(forward=options.Opts(spread_debug=True),
                              backward=options.Opts(debug=True))
    assert options.unpack_opts(opts, 1, True) == options.Opts(spread_debug=True)
    assert options.unpack_opts(opts, 1, False) == options.Opts(debug=True)


def test_nested_multi():
    opts = options.NestedOpts(
        forward=options.Opts(spread_debug=True),
        backward=options.NestedOpts(type1=options.Opts(spread_debug=True, debug=True),
                                    type2=options.Opts(debug=True)))
    assert options.unpack_opts(opts, 1, True) == options.Opts(spread_debug=True)
    assert options.unpack_opts(opts, 1, False) == options.NestedOpts(
        type1=options.Opts(spread_debug=True, debug=True), type2=options.Opts(debug=True))
    assert options.unpack_opts(options.unpack_opts(opts, 1, False), 1, True) == options.Opts(
        spread_debug=True, debug=True)
    assert options.unpack_opts(options.unpack_opts(opts, 1, False), 2, True) == options.Opts(
        debug=True)


def test_opts_validation_and_native():
    with pytest.raises(ValueError):
        options.Opts(gpu_upsampfac=1.0)
    with pytest.raises(ValueError):
        options.Opts(gpu_precision=7)
    n = options.to_native(options.Opts(modeord=True, gpu_method=2, gpu_binsizex=16,
                                       gpu_upsampfac=1.25))
    assert (n.modeord, n.gpu_method, n.gpu_binsizex, n.upsampfac) == (1, 2, 16, 1.25)
    o = options.Opts().to_cufinufft_opts()
    assert (o.upsampfac, o.gpu_method, o.gpu_sort, o.gpu_kerevalmeth) == (2.0, 0, 1, 1)
    assert hash(options.Opts()) == hash(options.Opts())


# --- the C ABI surface ----------------------------------------------------------
HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "gbnufft.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GBN_API\s+[\w\s\*]*?\b(gbnf?_\w+)\s*\(", text)))


def test_header_declares_full_abi():
    names = declared_symbols()
    for t in (1, 2, 3):
        for d in (1, 2, 3):
            assert "gbn_nufft%dd%df" % (d, t) in names
            assert "gbn_nufft%dd%d" % (d, t) in names
    for n in ("gbn_makeplan", "gbnf_makeplan", "gbn_setpts", "gbnf_setpts", "gbn_execute",
              "gbn_destroy", "gbn_run", "gbn_last_error", "gbn_default_opts"):
        assert n in names


def test_library_exports_every_declared_symbol(native):
    from jax_finufft_gb300 import _native

    for name in declared_symbols():
        assert hasattr(native, name), name
        assert name in _native.SIGNATURES, name


def test_default_opts_and_struct_layout(native):
    from jax_finufft_gb300 import _native

    o = _native.default_opts()
    assert (o.modeord, o.upsampfac, o.gpu_method, o.gpu_sort, o.gpu_kerevalmeth) == (
        0, 2.0, 0, 1, 1)
    assert o.gpu_maxsubprobsize == 1024 and o.gpu_precision == 0
    assert ctypes.sizeof(_native.GbnOpts) == 64


def test_cpu_tensors_are_rejected():
    """No CPU fallback: the product path refuses host tensors."""
    import jax_finufft_gb300 as jf

    x = torch.zeros(10, dtype=torch.float64)
    c = torch.zeros(10, dtype=torch.complex128)
    with pytest.raises(RuntimeError, match="CUDA"):
        jf.nufft1(8, c, x)


def _declared_arity():
    """Number of parameters of every GBN_API function, macros expanded."""
    text = open(HEADER).read()
    macros = {}
    for m in re.finditer(r"#define (GBN_ONESHOT_ARGS_[FD])((?:.*\\\n)*.*)", text):
        body = m.group(2).replace("\\\n", " ")
        macros[m.group(1)] = body.count(",") + 1
    out = {}
    for m in re.finditer(r"GBN_API\s+[\w\s\*]*?\b(gbnf?_\w+)\s*\(([^;]*?)\)\s*;", text, re.S):
        args = m.group(2).strip()
        if args in ("void", ""):
            out[m.group(1)] = 0
            continue
        n = 0
        for a in args.split(","):
            a = a.strip()
            n += macros.get(a, 1)
        out[m.group(1)] = n
    return out


def test_ctypes_arity_matches_header():
    from jax_finufft_gb300 import _native

    arity = _declared_arity()
    assert len(arity) == len(declared_symbols())
    for name, n in arity.items():
        assert len(_native.SIGNATURES[name][1]) == n, (name, n, len(_native.SIGNATURES[name][1]))


def test_xla_ffi_handlers_cover_the_targets():
    """The XLA FFI handler source defines one handler per one-shot entry point
    (the 18 targets of lib/jax_finufft_gpu.cc) and binds the attributes in
    the one-shot ABI's order."""
    import re

    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = open(os.path.join(repo, "jax-finufft_gb300", "xla", "gbn_xla_ffi.cc")).read()
    header = open(os.path.join(repo, "include", "gbnufft.h")).read()
    targets = re.findall(r"GBN_TARGET\((nufft\dd\df?),\s*(\d),\s*(\d),\s*(float|double)\)", src)
    names = {t[0] for t in targets}
    oneshot = set(re.findall(r"gbn_(nufft\dd\df?)\(", header))
    assert names == oneshot and len(names) == 18
    for name, dim, ty, eps in targets:
        assert name == "nufft%sd%s%s" % (dim, ty, "f" if eps == "float" else "")
    regs = set(re.findall(r"GBN_REG\((nufft\dd\df?)\)", src))
    assert regs == names
    attrs = re.findall(r'Attr<[^>]+>\("(\w+)"\)', src)
    assert attrs == ["eps", "iflag", "n_tot", "n_transf", "n_j", "n_k_1", "n_k_2", "n_k_3",
                     "modeord", "upsampfac", "gpu_method", "gpu_sort", "gpu_kerevalmeth",
                     "gpu_maxbatchsize", "debug"]
