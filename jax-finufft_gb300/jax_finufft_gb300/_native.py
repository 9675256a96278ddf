"""ctypes binding of libgbnufft.so (the C ABI in include/gbnufft.h).

This is the only route from Python to the GPU: there is no CPU fallback.
Loading fails with an error naming the build command when the library has
not been built.
"""
import ctypes
import os
import threading
import warnings

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgbnufft.so")

_lock = threading.Lock()
_lib = None

GBN_OK = 0
GBN_WARN_EPS_TOO_SMALL = 1


class NufftError(RuntimeError):
    """A non-zero error status from the native library."""

    def __init__(self, code, msg):
        super().__init__("gbnufft error %d: %s" % (code, msg))
        self.code = code


class GbnOpts(ctypes.Structure):
    """Mirror of ``struct gbn_opts``."""

    _fields_ = [
        ("modeord", ctypes.c_int),
        ("upsampfac", ctypes.c_double),
        ("gpu_method", ctypes.c_int),
        ("gpu_sort", ctypes.c_int),
        ("gpu_kerevalmeth", ctypes.c_int),
        ("gpu_maxbatchsize", ctypes.c_int),
        ("debug", ctypes.c_int),
        ("gpu_binsizex", ctypes.c_int),
        ("gpu_binsizey", ctypes.c_int),
        ("gpu_binsizez", ctypes.c_int),
        ("gpu_maxsubprobsize", ctypes.c_int),
        ("gpu_precision", ctypes.c_int),
        ("gpu_autotune", ctypes.c_int),
        ("gpu_kernel", ctypes.c_int),
    ]


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i64p = ctypes.POINTER(ctypes.c_int64)

# Every symbol include/gbnufft.h declares, with its argument types.
# stream, eps, then iflag n_tot n_transf n_j n_k_1 n_k_2 n_k_3 modeord, upsampfac,
# then gpu_method gpu_sort gpu_kerevalmeth gpu_maxbatchsize debug
_ONESHOT_F = [_vp, ctypes.c_float] + [_i64] * 8 + [ctypes.c_double] + [_i64] * 5
_ONESHOT_D = [_vp, ctypes.c_double] + [_i64] * 8 + [ctypes.c_double] + [_i64] * 5
SIGNATURES = {
    "gbn_default_opts": (None, [ctypes.POINTER(GbnOpts)]),
    "gbn_makeplan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _i64p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.POINTER(_vp),
                                    ctypes.POINTER(GbnOpts), _vp]),
    "gbnf_makeplan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _i64p, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_float, ctypes.POINTER(_vp),
                                     ctypes.POINTER(GbnOpts), _vp]),
    "gbn_setpts": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "gbnf_setpts": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "gbn_execute": (ctypes.c_int, [_vp, _vp, _vp]),
    "gbn_set_stream": (ctypes.c_int, [_vp, _vp]),
    "gbn_destroy": (ctypes.c_int, [_vp]),
    "gbn_plan_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), _i64p,
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "gbn_get_timings": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_int)]),
    "gbn_debug_bins": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p]),
    "gbn_debug_fold": (ctypes.c_int, [_vp, _i64p, ctypes.POINTER(ctypes.c_double)]),
    "gbn_last_error": (ctypes.c_char_p, []),
    "gbn_clear_cache": (None, []),
    "gbn_launch_count": (ctypes.c_longlong, []),
    "gbn_points_create": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "gbn_points_destroy": (ctypes.c_int, [_vp]),
    "gbn_execute_points": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "gbn_grad": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "gbn_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        _i64p, _i64p, ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.POINTER(GbnOpts), _vp, ctypes.POINTER(_vp)]),
    "gbn_batch_run": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int]),
    "gbn_batch_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int), _i64p]),
    "gbn_batch_destroy": (ctypes.c_int, [_vp]),
    "gbn_batch_chain_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _vp,
                                              ctypes.POINTER(_vp)]),
    "gbn_batch_chain_run": (ctypes.c_int, [_vp] + [ctypes.POINTER(_vp)] * 5 + [ctypes.c_int]),
    "gbn_batch_chain_destroy": (ctypes.c_int, [_vp]),
    "gbn_autotune": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i64p, _i64,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_int, _vp, _vp, _vp,
                                    _vp]),
    "gbn_autotune_clear": (None, [ctypes.c_int]),
    "gbn_wait_timeouts": (ctypes.c_int, [ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "gbn_set_t3_extents": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_double)] * 4),
    "gbn_debug_raise_wait_timeout": (None, []),
    "gbn_binsort_noalloc": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _i64, _vp, _vp, _vp,
                                           _i64p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                           _vp, _vp, _vp]),
    "gbn_run": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_double,
                               ctypes.c_int, _i64, _i64, _i64, _i64p, ctypes.POINTER(GbnOpts),
                               _vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _vp]),
}
for _t in (1, 2, 3):
    for _d in (1, 2, 3):
        _np = _d if _t != 3 else 2 * _d
        SIGNATURES["gbn_nufft%dd%df" % (_d, _t)] = (ctypes.c_int, _ONESHOT_F + [_vp] * (_np + 2))
        SIGNATURES["gbn_nufft%dd%d" % (_d, _t)] = (ctypes.c_int, _ONESHOT_D + [_vp] * (_np + 2))


def load(path=None):
    """Load libgbnufft.so and declare every exported function."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                "libgbnufft.so is not built (%s). Build it with "
                "`python jax-finufft_gb300/build.py` (needs nvcc with sm_103a support)." % p)
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def last_error():
    return load().gbn_last_error().decode(errors="replace")


def check(rc, what="call"):
    """Raise on an error status, warn on the tolerance warning."""
    if rc == GBN_OK:
        return
    if rc == GBN_WARN_EPS_TOO_SMALL:
        warnings.warn("%s: requested tolerance is not reachable; it was clamped" % what,
                      RuntimeWarning, stacklevel=3)
        return
    raise NufftError(rc, last_error())


def default_opts():
    o = GbnOpts()
    load().gbn_default_opts(ctypes.byref(o))
    return o


def run(nufft_type, dim, single, stream, eps, iflag, n_tot, n_transf, n_j, n_k, opts, source,
        pts, tgts, output):
    """Call gbn_run with raw device pointers (ints) and a GbnOpts."""
    lib = load()
    nk = (ctypes.c_int64 * 3)(*[int(v) for v in n_k])
    P = (_vp * 3)(*[_vp(int(p)) if p else None for p in list(pts) + [0] * (3 - len(pts))])
    T = (_vp * 3)(*[_vp(int(p)) if p else None for p in list(tgts) + [0] * (3 - len(tgts))])
    rc = lib.gbn_run(int(nufft_type), int(dim), int(bool(single)), _vp(int(stream) or None),
                     float(eps), int(iflag), int(n_tot), int(n_transf), int(n_j), nk,
                     ctypes.byref(opts), _vp(int(source) or None), P, T,
                     _vp(int(output) or None))
    check(rc, "nufft%d" % nufft_type)
    return rc
