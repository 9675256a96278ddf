"""Options with the field names, defaults and nesting rules of
src/jax_finufft/options.py (Opts :46-119, NestedOpts :122-129,
unpack_opts :132-148).

The reference builds these with pydantic; plain frozen dataclasses are used
here (pydantic is not available everywhere this package runs), keeping
equality, hashing and keyword construction identical.  Only the GPU fields
and ``modeord`` reach the GB300 engine (as in ``to_cufinufft_opts``,
options.py:105-119), plus the bin-size / subproblem fields that the reference
carries but never forwards, and the engine's own fields: ``gpu_precision`` (compute precision; 0 = the
data's, the reference behaviour), ``gpu_fused_adjoint``, ``gpu_autotune`` and
``gpu_kernel`` (spreading kernel shape: 0 the exponential of semicircle, the
reference's; 1 Kaiser-Bessel, more accurate at the same width).
"""
from dataclasses import dataclass
from enum import IntEnum
from typing import Optional, Union

# FFTW planner flags (FFTW's public values), kept for CPU-field parity.
FFTW_ESTIMATE = 1 << 6
FFTW_MEASURE = 0
FFTW_PATIENT = 1 << 5
FFTW_EXHAUSTIVE = 1 << 3
FFTW_WISDOM_ONLY = 1 << 21


class DebugLevel(IntEnum):
    Silent = 0
    Verbose = 1
    Noisy = 2


class GpuDebugLevel(IntEnum):
    Silent = 0
    Verbose = 1


class FftwFlags(IntEnum):
    Estimate = FFTW_ESTIMATE
    Measure = FFTW_MEASURE
    Patient = FFTW_PATIENT
    Exhaustive = FFTW_EXHAUSTIVE
    WisdomOnly = FFTW_WISDOM_ONLY


class SpreadSort(IntEnum):
    NoSort = 0
    Sort = 1
    Heuristic = 2


class SpreadThread(IntEnum):
    Auto = 0
    Sequential = 1
    Parallel = 2


class GpuKernel(IntEnum):
    ExponentialOfSemicircle = 0
    KaiserBessel = 1


class GpuMethod(IntEnum):
    Auto = 0
    Driven = 1
    Shared = 2


class GpuPrecision(IntEnum):
    Data = 0  # complex64 -> FP32, complex128 -> FP64 (the reference's behaviour)
    Single = 1
    Double = 2
    Split = 3  # FP32 when eps >= 1e-6, FP64 otherwise


@dataclass(frozen=True)
class Opts:
    # CPU (FINUFFT) fields: accepted for API parity, unused by the GPU engine.
    modeord: bool = False
    debug: DebugLevel = DebugLevel.Silent
    spread_debug: DebugLevel = DebugLevel.Silent
    showwarn: bool = False
    nthreads: int = 0
    fftw: int = FftwFlags.Estimate
    spread_sort: SpreadSort = SpreadSort.Heuristic
    spread_kerevalmeth: bool = True
    spread_kerpad: bool = True
    upsampfac: float = 0.0
    spread_thread: SpreadThread = SpreadThread.Auto
    maxbatchsize: int = 0
    spread_nthr_atomic: int = -1
    spread_max_sp_size: int = 0

    # GPU fields (cuFINUFFT's defaults).
    gpu_upsampfac: float = 2.0
    gpu_method: GpuMethod = 0
    gpu_sort: bool = True
    gpu_binsizex: int = 0
    gpu_binsizey: int = 0
    gpu_binsizez: int = 0
    gpu_obinsizex: int = 0
    gpu_obinsizey: int = 0
    gpu_obinsizez: int = 0
    gpu_maxsubprobsize: int = 1024
    gpu_kerevalmeth: bool = True
    gpu_spreadinterponly: bool = False
    gpu_maxbatchsize: int = 0
    gpu_debug: GpuDebugLevel = GpuDebugLevel.Silent

    # GB300 engine extensions.
    gpu_precision: GpuPrecision = 0
    # reverse mode through one fused adjoint on the forward's sorted points
    # (False: the stacked-transform rules of the reference's JVP/transpose)
    gpu_fused_adjoint: bool = True
    # types 1/2: look up (or tune, on a cache miss) sigma, method, bin sizes
    # and points per subproblem for each call's class (see tune.py)
    gpu_autotune: bool = False
    # spreading kernel: 0 exponential of semicircle (FINUFFT's), 1 Kaiser-Bessel
    # (same width rule and cost, 1.5-2.5x smaller aliasing error)
    gpu_kernel: GpuKernel = 0

    def __post_init__(self):
        if int(self.modeord) not in (0, 1):
            raise ValueError("modeord must be 0 or 1")
        if not float(self.gpu_upsampfac) > 1.0:
            raise ValueError("gpu_upsampfac must be > 1")
        if int(self.gpu_method) not in (0, 1, 2):
            raise ValueError("gpu_method must be 0, 1 or 2")
        if int(self.gpu_precision) not in (0, 1, 2, 3):
            raise ValueError("gpu_precision must be 0..3")
        if int(self.gpu_kernel) not in (0, 1):
            raise ValueError("gpu_kernel must be 0 (exponential of semicircle) or 1 (Kaiser-Bessel)")
        if self.gpu_spreadinterponly:
            raise ValueError("gpu_spreadinterponly is not supported")

    def to_cufinufft_opts(self):
        """The seven GPU attributes the reference forwards (options.py:105-119)."""

        class NativeOpts:
            pass

        opts = NativeOpts()
        opts.modeord = int(self.modeord)
        opts.upsampfac = float(self.gpu_upsampfac)
        opts.gpu_method = int(self.gpu_method)
        opts.gpu_sort = int(self.gpu_sort)
        opts.gpu_kerevalmeth = int(self.gpu_kerevalmeth)
        opts.gpu_maxbatchsize = int(self.gpu_maxbatchsize)
        opts.debug = int(self.gpu_debug)
        return opts


@dataclass(frozen=True)
class NestedOpts:
    type1: Optional[Opts] = None
    type2: Optional[Opts] = None
    type3: Optional[Opts] = None

    forward: Optional[Opts] = None
    backward: Optional[Union[Opts, "NestedOpts"]] = None


def unpack_opts(opts, finufft_type, forward):
    """Pick the options for one transform (options.py:132-148)."""
    if opts is None or isinstance(opts, Opts):
        return opts

    if forward:
        if opts.forward is not None:
            return opts.forward
        elif finufft_type == 1:
            return opts.type1
        elif finufft_type == 2:
            return opts.type2
        elif finufft_type == 3:
            return opts.type3
    elif opts.backward is not None:
        return opts.backward

    return opts


def to_native(opts):
    """Opts (or None) -> the C struct gbn_opts."""
    from ._native import GbnOpts

    o = opts if opts is not None else Opts()
    n = GbnOpts()
    n.modeord = int(o.modeord)
    n.upsampfac = float(o.gpu_upsampfac)
    n.gpu_method = int(o.gpu_method)
    n.gpu_sort = int(bool(o.gpu_sort))
    n.gpu_kerevalmeth = int(bool(o.gpu_kerevalmeth))
    n.gpu_maxbatchsize = int(o.gpu_maxbatchsize)
    n.debug = int(o.gpu_debug)
    n.gpu_binsizex = int(o.gpu_binsizex)
    n.gpu_binsizey = int(o.gpu_binsizey)
    n.gpu_binsizez = int(o.gpu_binsizez)
    n.gpu_maxsubprobsize = int(o.gpu_maxsubprobsize)
    n.gpu_precision = int(o.gpu_precision)
    n.gpu_kernel = int(o.gpu_kernel)
    return n
