"""GB300-native NUFFT behind jax-finufft's nufft1/nufft2/nufft3 API.

The transforms run in libgbnufft.so (hand-written sm_103a kernels plus cuFFT)
through its C ABI; this package is the PyTorch host mirror of the reference's
Python interface (src/jax_finufft/__init__.py:15-18).
"""
__version__ = "0.1.0"
__all__ = ["__version__", "nufft1", "nufft2", "nufft3"]

from .ops import nufft1, nufft2, nufft3  # noqa: E402
