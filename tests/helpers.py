"""Shared helpers for the tests (tolerances follow the reference's tests)."""
import numpy as np

# tests/ops_test.py:14-16 -- rtol per output dtype; atol from jax's defaults
RTOL = {"complex128": 1e-7, "complex64": 1e-4, "float64": 1e-7, "float32": 1e-4}
ATOL = {"complex128": 1e-15, "complex64": 1e-6, "float64": 1e-15, "float32": 1e-6}


def check_close(actual, expected, rtol=None, dtype=None, floor=True):
    """Elementwise |a - b| <= atol + rtol*|b| (jax test_util.check_close).

    With ``floor`` the absolute tolerance is raised to 1e-2*rtol*rms(|b|):
    entries a hundred times smaller than typical are held to an absolute
    rather than a relative bound, since a NUFFT's error is spread evenly over
    the modes (relative-l2 accuracy ~ eps), not proportional to each entry.
    The relative-l2 error itself is checked against rtol as well.
    """
    a = np.asarray(actual)
    b = np.asarray(expected)
    key = str(dtype or a.dtype)
    if rtol is None:
        rtol = RTOL[key]
    elif isinstance(rtol, dict):
        rtol = rtol[key]
    atol = ATOL.get(key, 0.0)
    if floor and b.size:
        atol = max(atol, 1e-2 * rtol * float(np.sqrt(np.mean(np.abs(b) ** 2))))
        assert rel_l2(a, b) <= rtol, (rel_l2(a, b), rtol)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def golden(name):
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name)
    return np.load(here)
