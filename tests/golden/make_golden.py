"""Generate the golden known-answer fixtures under tests/golden/.

The reference's tests (tests/ops_test.py) draw their inputs from
``np.random.default_rng(seed)`` and compare each transform with a direct
NUDFT sum computed in the test.  This script replays those draws in the same
order for the same parameter grids and stores inputs and the FP64 direct-sum
answers, so the oracle and the CUDA path are both checked against the
reference tests' own known answers without jax:

  forward.npz  -- test_nufft1_forward / test_nufft2_forward (ops_test.py:25-93):
                  ndim 1..3, x64 False/True, M=50, modes 75//ndim + 5*arange,
                  iflag -1/+1, seed 657
                  test_nufft3_forward (ops_test.py:96-125): 25 sources,
                  20 targets in [-1, 1), seed 657
  modeord.npz  -- test_modeord (ops_test.py:494-567): modeord 0/1,
                  Nf 16/17, ndim 1..3, types 1/2, iflag +1, seed 657
  multi.npz    -- test_multi_transform (ops_test.py:380-397): seed 314,
                  n_tot=5, n_tr=1, n_j=50, n_k=12, 35 targets

Expected values are complex128 direct sums over the (possibly float32-cast)
inputs.  Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys
from itertools import product

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import direct  # noqa: E402


def forward():
    out = {}
    for ndim, x64, iflag in product([1, 2, 3], [False, True], [-1, 1]):
        dtype = np.double if x64 else np.single
        cdtype = np.cdouble if x64 else np.csingle
        key = "d%d_%s_i%+d" % (ndim, "x64" if x64 else "x32", iflag)
        nu = tuple(int(v) for v in 75 // ndim + 5 * np.arange(ndim))
        # type 1
        rng = np.random.default_rng(657)
        x = rng.uniform(-np.pi, np.pi, size=(ndim, 50)).astype(dtype)
        c = rng.normal(size=50) + 1j * rng.normal(size=50)
        c = c.astype(cdtype)
        out["t1_" + key + "_x"] = x
        out["t1_" + key + "_c"] = c
        out["t1_" + key + "_f"] = direct.type1(c, list(x), nu, iflag)
        # type 2
        rng = np.random.default_rng(657)
        xs = np.stack([rng.uniform(-np.pi, np.pi, size=50).astype(dtype) for _ in range(ndim)])
        f = rng.normal(size=nu) + 1j * rng.normal(size=nu)
        f = f.astype(cdtype)
        out["t2_" + key + "_x"] = xs
        out["t2_" + key + "_f"] = f
        out["t2_" + key + "_c"] = direct.type2(f, list(xs), iflag)
        # type 3
        rng = np.random.default_rng(657)
        xs = np.stack([rng.uniform(-1.0, 1.0, size=25).astype(dtype) for _ in range(ndim)])
        ss = np.stack([rng.uniform(-1.0, 1.0, size=20).astype(dtype) for _ in range(ndim)])
        c = rng.normal(size=25) + 1j * rng.normal(size=25)
        c = c.astype(cdtype)
        out["t3_" + key + "_x"] = xs
        out["t3_" + key + "_s"] = ss
        out["t3_" + key + "_c"] = c
        out["t3_" + key + "_f"] = direct.type3(c, list(xs), list(ss), iflag)
    return out


def modeord():
    out = {}
    for mo, nf, ndim, ty in product([0, 1], [16, 17], [1, 2, 3], [1, 2]):
        rng = np.random.default_rng(657)
        nu = tuple(int(v) for v in nf // ndim + 5 * np.arange(ndim))
        key = "mo%d_n%d_d%d_t%d" % (mo, nf, ndim, ty)
        x = rng.uniform(-np.pi, np.pi, size=(ndim, 50)).astype(np.double)
        if ty == 1:
            c = rng.normal(size=50) + 1j * rng.normal(size=50)
            out[key + "_x"] = x
            out[key + "_c"] = c
            out[key + "_f"] = direct.type1(c, list(x), nu, 1, modeord=mo)
        else:
            f = rng.normal(size=nu) + 1j * rng.normal(size=nu)
            out[key + "_x"] = x
            out[key + "_f"] = f
            out[key + "_c"] = direct.type2(f, list(x), 1, modeord=mo)
    return out


def multi():
    rng = np.random.default_rng(314)
    n_tot, n_tr, n_j, n_k, n_target = 5, 1, 50, 12, 35
    f = rng.standard_normal(size=(n_tot, n_tr, n_k)) + 1j * rng.standard_normal(
        size=(n_tot, n_tr, n_k))
    c = rng.standard_normal(size=(n_tot, n_tr, n_j)) + 1j * rng.standard_normal(
        size=(n_tot, n_tr, n_j))
    x = rng.uniform(-np.pi, np.pi, (n_tot, n_j))
    xt = rng.uniform(-1.0, 1.0, (n_tot, n_target))
    e1 = np.zeros((n_tot, n_tr, n_k), complex)
    e2 = np.zeros((n_tot, n_tr, n_j), complex)
    e3 = np.zeros((n_tot, n_tr, n_target), complex)
    for i in range(n_tot):
        for t in range(n_tr):
            e1[i, t] = direct.type1(c[i, t], [x[i]], (n_k,), 1)
            e2[i, t] = direct.type2(f[i, t], [x[i]], -1)
            e3[i, t] = direct.type3(c[i, t], [x[i]], [xt[i]], -1)
    return dict(f=f, c=c, x=x, xt=xt, t1=e1, t2=e2, t3=e3, n_k=np.array(n_k))


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "forward.npz"), **forward())
    np.savez_compressed(os.path.join(HERE, "modeord.npz"), **modeord())
    np.savez_compressed(os.path.join(HERE, "multi.npz"), **multi())
    for n in ("forward.npz", "modeord.npz", "multi.npz"):
        print(n, os.path.getsize(os.path.join(HERE, n)))
