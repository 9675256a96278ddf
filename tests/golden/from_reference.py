"""Golden fixtures computed by the reference's own test code.

The reference's tests (tests/ops_test.py of jax-finufft) compute their known
answers with plain numpy inside the test functions -- the direct NUDFT sums
of test_nufft{1,2,3}_forward (ops_test.py:25-125) and test_modeord
(ops_test.py:494-567) -- and then compare the library's output with them.
This script executes that test file as written, with ``jax``,
``jax.numpy``, ``jax._src.test_util`` and ``jax_finufft`` replaced by
stand-ins that record each call instead of transforming: the stand-in
``nufft1/2/3`` returns a record of its arguments, and the stand-in
``check_close`` stores (record, expected, rtol).  Every test of the
reference's parameter grids (read from its own ``pytest.mark.parametrize``
marks) is run once; the first comparison of each test gives the fixture:

  forward.npz  keys t{1,2,3}_d{ndim}_{x32,x64}_i{+1,-1}_{x,c,f[,s]}
  modeord.npz  keys mo{0,1}_n{16,17}_d{ndim}_t{1,2}_{x,c,f}
  multi.npz    test_multi_transform (ops_test.py:380-397) has no known
               answer of its own (it compares the n_tot path with per-slice
               calls), so its inputs are recorded from the test and the
               expected values are FP64 direct sums from oracle/direct.py

Expected arrays keep the dtype the reference computed them in (complex64 for
the float32 cases: the test accumulates in complex128 and stores into a
complex64 array).  The reference sources are only needed to regenerate:

  python tests/golden/from_reference.py [--ref /root/reference]

The fixtures are committed; nothing at test time reads the reference.
"""
import argparse
import contextlib
import importlib.util
import itertools
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


class Call:
    """What a stand-in transform was called with."""

    def __init__(self, name, args, kwargs):
        self.name, self.args, self.kwargs = name, args, kwargs

    def __getitem__(self, index):  # calc[:, n] in test_multi_transform
        return self


class Recorder:
    def __init__(self):
        self.records = []

    def check_close(self, a, b, atol=None, rtol=None, err_msg=""):
        self.records.append((a, b, rtol))

    def take(self):
        r, self.records = self.records, []
        return r


def install_stubs(rec):
    """Stand-in modules for everything ops_test.py imports besides numpy,
    pytest and the standard library."""
    def passthrough(fn=None, *a, **k):
        return fn

    jax = types.ModuleType("jax")
    jax.version = types.SimpleNamespace(__version_info__=(0, 8, 0))
    jax.enable_x64 = lambda *a, **k: contextlib.nullcontext()
    jax.jit = passthrough
    jax.experimental = types.SimpleNamespace(enable_x64=jax.enable_x64)

    def unsupported(*a, **k):
        raise RuntimeError("this test needs jax itself; only known-answer tests are replayed")

    jax.vmap = jax.grad = jax.jvp = unsupported
    jnp = types.ModuleType("jax.numpy")
    jnp.__getattr__ = lambda name: getattr(np, name)
    jax.numpy = jnp
    src = types.ModuleType("jax._src")
    tu = types.ModuleType("jax._src.test_util")
    tu.check_close = rec.check_close
    tu.check_grads = lambda *a, **k: None
    src.test_util = tu
    jax._src = src

    jf = types.ModuleType("jax_finufft")
    for name in ("nufft1", "nufft2", "nufft3"):
        setattr(jf, name, (lambda n: lambda *a, **k: Call(n, a, k))(name))
    jfo = types.ModuleType("jax_finufft.options")
    jfo.Opts = lambda **k: types.SimpleNamespace(**k)
    jf.options = jfo
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "jax._src": src,
                        "jax._src.test_util": tu, "jax_finufft": jf,
                        "jax_finufft.options": jfo})


def load_reference_tests(ref):
    path = os.path.join(ref, "tests", "ops_test.py")
    spec = importlib.util.spec_from_file_location("reference_ops_test", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def param_grid(fn):
    """Keyword sets of a test's stacked pytest.mark.parametrize marks, in the
    order pytest generates them."""
    axes = []
    for m in getattr(fn, "pytestmark", []):
        if m.name != "parametrize":
            continue
        names = [s.strip() for s in m.args[0].split(",")]
        vals = list(m.args[1])
        axes.append([dict(zip(names, v if len(names) > 1 else (v,))) for v in vals])
    for combo in itertools.product(*reversed(axes)):
        kw = {}
        for part in combo:
            kw.update(part)
        yield kw


def first(rec, name):
    r = rec.take()
    call, expect, rtol = r[0]
    assert isinstance(call, Call) and call.name == name, (call, name)
    return call, np.asarray(expect), rtol


def forward(mod, rec):
    out = {}
    for kw in param_grid(mod.test_nufft1_forward):
        mod.test_nufft1_forward(**kw)
        call, f, _ = first(rec, "nufft1")
        ndim = kw["ndim"]
        key = "t1_d%d_%s_i%+d" % (ndim, "x64" if kw["x64"] else "x32", kw["iflag"])
        shape, c, xs = call.args[0], call.args[1], call.args[2:]
        assert tuple(f.shape) == tuple(int(n) for n in shape) and len(xs) == ndim
        out[key + "_x"] = np.stack(xs)
        out[key + "_c"] = np.asarray(c)
        out[key + "_f"] = f
    for kw in param_grid(mod.test_nufft2_forward):
        mod.test_nufft2_forward(**kw)
        call, c, _ = first(rec, "nufft2")
        key = "t2_d%d_%s_i%+d" % (kw["ndim"], "x64" if kw["x64"] else "x32", kw["iflag"])
        out[key + "_x"] = np.stack(call.args[1:])
        out[key + "_f"] = np.asarray(call.args[0])
        out[key + "_c"] = c
    for kw in param_grid(mod.test_nufft3_forward):
        mod.test_nufft3_forward(**kw)
        call, f, rtol = first(rec, "nufft3")
        ndim = kw["ndim"]
        key = "t3_d%d_%s_i%+d" % (ndim, "x64" if kw["x64"] else "x32", kw["iflag"])
        pts = call.args[1:]
        out[key + "_x"] = np.stack(pts[:ndim])
        out[key + "_s"] = np.stack(pts[ndim:])
        out[key + "_c"] = np.asarray(call.args[0])
        out[key + "_f"] = f
        out["t3_rtol_complex64"] = np.array(rtol["complex64"])
        out["t3_rtol_complex128"] = np.array(rtol["complex128"])
    return out


def modeord(mod, rec):
    out = {}
    for kw in param_grid(mod.test_modeord):
        mod.test_modeord(**kw)
        ty = kw["nufft_type"]
        key = "mo%d_n%d_d%d_t%d" % (kw["modeord"], kw["Nf"], kw["ndim"], ty)
        call, expect, _ = first(rec, "nufft%d" % ty)
        assert call.kwargs["opts"].modeord == kw["modeord"]
        if ty == 1:
            out[key + "_x"] = np.stack(call.args[2:])
            out[key + "_c"] = np.asarray(call.args[1])
            out[key + "_f"] = expect
        else:
            out[key + "_x"] = np.stack(call.args[1:])
            out[key + "_f"] = np.asarray(call.args[0])
            out[key + "_c"] = expect
    return out


def multi(mod, rec):
    sys.path.insert(0, REPO)
    from oracle import direct

    mod.test_multi_transform()
    r = rec.take()
    c1 = r[0][0]  # nufft1(n_k, c, x)
    c2 = r[1][0]  # nufft2(f, x)
    c3 = r[2][0]  # nufft3(c, x, x_target)
    n_k, c, x = c1.args
    f = c2.args[0]
    xt = c3.args[2]
    n_tot, n_tr = c.shape[:2]
    e1 = np.zeros((n_tot, n_tr, n_k), complex)
    e2 = np.zeros((n_tot, n_tr, x.shape[1]), complex)
    e3 = np.zeros((n_tot, n_tr, xt.shape[1]), complex)
    # the test passes no iflag: the defaults of src/jax_finufft/ops.py:51, 86,
    # 127 apply (type 1: +1, types 2 and 3: -1)
    assert not (c1.kwargs or c2.kwargs or c3.kwargs)
    for i in range(n_tot):
        for t in range(n_tr):
            e1[i, t] = direct.type1(c[i, t], [x[i]], (n_k,), 1)
            e2[i, t] = direct.type2(f[i, t], [x[i]], -1)
            e3[i, t] = direct.type3(c[i, t], [x[i]], [xt[i]], -1)
    return dict(f=f, c=c, x=x, xt=xt, t1=e1, t2=e2, t3=e3, n_k=np.array(n_k))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference",
                    help="checkout of jax-finufft whose tests/ops_test.py is replayed")
    args = ap.parse_args()
    rec = Recorder()
    install_stubs(rec)
    mod = load_reference_tests(args.ref)
    files = {"forward.npz": forward(mod, rec), "modeord.npz": modeord(mod, rec),
             "multi.npz": multi(mod, rec)}
    for name, arrays in files.items():
        np.savez_compressed(os.path.join(HERE, name), **arrays)
        print(name, len(arrays), "arrays", os.path.getsize(os.path.join(HERE, name)), "bytes")


if __name__ == "__main__":
    main()
