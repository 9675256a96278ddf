"""FP64 direct NUDFT sums -- the known-answer oracle (test infrastructure only).

These are the sums the reference's own tests compare against:
  type 1  f_k = sum_j c_j exp(iflag*i*k.x_j)   (tests/ops_test.py:42-45)
  type 2  c_j = sum_k f_k exp(iflag*i*k.x_j)   (tests/ops_test.py:77-84)
  type 3  f_k = sum_j c_j exp(iflag*i*s_k.x_j) (tests/ops_test.py:112-116)
with k ranging over src/jax_finufft/ops.py:114-123 ``get_frequency_array``.
Axes are in the user's order: point array ``a`` pairs with mode axis ``a``.
All arithmetic is complex128; the sums are contracted one axis at a time and
chunked over points so bench-sized subsets stay within memory.
"""
import numpy as np


def frequencies(n, modeord=0):
    """Integer frequencies of the n modes of one axis in storage order."""
    n = int(n)
    if modeord == 0:
        return np.arange(-(n // 2), (n + 1) // 2, dtype=np.int64)
    if modeord == 1:
        f = np.empty(n, dtype=np.int64)
        f[: (n + 1) // 2] = np.arange(0, (n + 1) // 2)
        f[(n + 1) // 2:] = np.arange(-(n // 2), 0)
        return f
    raise ValueError("Unsupported modeord: %r" % (modeord,))


def _as_c128(a):
    return np.asarray(a).astype(np.complex128)


def type1(c, points, n_modes=None, iflag=1, modeord=0, ks=None, chunk=1 << 16):
    """f[k_0, ..., k_{d-1}] for one transform (c of shape (M,)).

    ``ks`` optionally gives, per axis, the integer frequencies to evaluate
    (a sub-grid of modes); otherwise all modes of ``n_modes`` in ``modeord``
    order.
    """
    c = _as_c128(c)
    pts = [np.asarray(p, dtype=np.float64) for p in points]
    d = len(pts)
    if ks is None:
        ks = [frequencies(n, modeord) for n in n_modes]
    ks = [np.asarray(k, dtype=np.float64) for k in ks]
    shape = tuple(len(k) for k in ks)
    out = np.zeros(shape, dtype=np.complex128)
    M = c.shape[0]
    for lo in range(0, M, chunk):
        hi = min(M, lo + chunk)
        E = [np.exp(1j * iflag * np.outer(ks[a], pts[a][lo:hi])) for a in range(d)]
        acc = E[0] * c[lo:hi][None, :]
        for a in range(1, d):
            # acc: (n_0*...*n_{a-1}, m)  x  E[a]: (n_a, m)
            if a == d - 1:
                out += (acc @ E[a].T).reshape(shape)
            else:
                acc = (acc[:, None, :] * E[a][None, :, :]).reshape(-1, hi - lo)
        if d == 1:
            out += acc.sum(axis=1)
    return out


def type2(f, points, iflag=-1, modeord=0, chunk=256):
    """c_j for one transform (f of shape (N_0, ..., N_{d-1}))."""
    f = _as_c128(f)
    pts = [np.asarray(p, dtype=np.float64) for p in points]
    d = len(pts)
    ks = [frequencies(n, modeord).astype(np.float64) for n in f.shape]
    M = pts[0].shape[0]
    out = np.zeros(M, dtype=np.complex128)
    for lo in range(0, M, chunk):
        hi = min(M, lo + chunk)
        # contract the last axis first: g[..., j]
        E = np.exp(1j * iflag * np.outer(ks[d - 1], pts[d - 1][lo:hi]))  # (N_last, m)
        g = np.tensordot(f, E, axes=([d - 1], [0]))  # (N_0..N_{d-2}, m)
        for a in range(d - 2, -1, -1):
            Ea = np.exp(1j * iflag * np.outer(ks[a], pts[a][lo:hi]))  # (N_a, m)
            shp = [1] * (a + 2)
            shp[a] = Ea.shape[0]
            shp[-1] = hi - lo
            g = (g * Ea.reshape(shp)).sum(axis=a)
        out[lo:hi] = g
    return out


def type3(c, sources, targets, iflag=-1, chunk=2048):
    """f_k = sum_j c_j exp(iflag*i*s_k.x_j) for one transform."""
    c = _as_c128(c)
    xs = [np.asarray(p, dtype=np.float64) for p in sources]
    ss = [np.asarray(p, dtype=np.float64) for p in targets]
    K = ss[0].shape[0]
    out = np.zeros(K, dtype=np.complex128)
    for lo in range(0, K, chunk):
        hi = min(K, lo + chunk)
        ph = np.zeros((hi - lo, c.shape[0]))
        for x, s in zip(xs, ss):
            ph += np.outer(s[lo:hi], x)
        out[lo:hi] = np.exp(1j * iflag * ph) @ c
    return out


def rel_l2(a, b):
    """Relative l2 error ||a - b|| / ||b||."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return float(num / den) if den > 0 else float(num)
