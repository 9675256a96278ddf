"""Build libgbnufft.so, the sm_103a NUFFT library, in-tree.

    python jax-finufft_gb300/build.py [-v] [--force]

Compiles each translation unit of csrc/ with nvcc for sm_103a in parallel and
links them with cuFFT into jax_finufft_gb300/_lib/libgbnufft.so.  A stamp file
holding a hash of the sources and flags lets repeated calls skip the build.
No cmake, no torch extension machinery: the library has a pure C ABI
(include/gbnufft.h) and is loaded with ctypes.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(HERE, "jax_finufft_gb300", "_lib")
BUILD_DIR = os.path.join(OUT_DIR, "obj")
LIB_NAME = "libgbnufft.so"

SOURCES = ["gbn_setpts.cu", "gbn_spread.cu", "gbn_interp.cu", "gbn_grad.cu", "gbn_plan.cu",
           "gbn_fft.cu", "gbn_tune.cu", "gbn_noalloc.cu"]
# bench.py's shared-memory atomic probe: a library of its own
PROBE_SRC = os.path.join(HERE, "bench_probe", "gbn_probe.cu")
PROBE_LIB = "libgbnprobe.so"
HEADERS = ["gbn_common.cuh", "gbn_device.cuh", "gbn_fold.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE,
                     "-diag-suppress", "128"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbnufft.so")


def cuda_lib_dir():
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for sub in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
                os.path.join("targets", "x86_64-linux", "lib")):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcufft.so")):
            return d
    return os.path.join(root, "lib64")


def library_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def probe_library_path():
    return os.path.join(OUT_DIR, PROBE_LIB)


def _stamp():
    h = hashlib.sha256()
    for name in SOURCES + HEADERS:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + f.read())
    with open(PROBE_SRC, "rb") as f:
        h.update(f.read())
    with open(os.path.join(INCLUDE, "gbnufft.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def up_to_date():
    stamp = os.path.join(OUT_DIR, "stamp.txt")
    if not (os.path.exists(library_path()) and os.path.exists(stamp) and
            os.path.exists(probe_library_path())):
        return False
    with open(stamp) as f:
        return f.read().strip() == _stamp()


def build(verbose=False, force=False):
    if not force and up_to_date():
        return library_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    exe = nvcc()

    def compile_one(name):
        obj = os.path.join(BUILD_DIR, name.replace(".cu", ".o"))
        cmd = [exe] + NVCC_FLAGS + ["-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (name, r.stdout, r.stderr))
        if r.stderr.strip():
            print(r.stderr, file=sys.stderr, flush=True)  # warnings
        return obj

    def build_probe():
        tmp = probe_library_path() + ".tmp%d" % os.getpid()
        cmd = [exe] + ARCH + ["-O3", "-Xcompiler", "-fPIC", "-shared", PROBE_SRC, "-o", tmp]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for the probe:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, probe_library_path())

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        probe = ex.submit(build_probe)
        objs = list(ex.map(compile_one, SOURCES))
        probe.result()
    libdir = cuda_lib_dir()
    tmp = library_path() + ".tmp%d" % os.getpid()
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-L" + libdir, "-lcufft", "-Xlinker", "-rpath=" + libdir]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, library_path())
    with open(os.path.join(OUT_DIR, "stamp.txt"), "w") as f:
        f.write(_stamp())
    return library_path()


def build_xla_ffi(verbose=False):
    """Compile xla/gbn_xla_ffi.cc into the module jax_finufft_gpu (the XLA
    FFI handlers jax-finufft's lowering registers) next to libgbnufft.so.
    Needs jax (for the FFI headers) and pybind11; returns the module path,
    or None when either is missing."""
    try:
        import jax.ffi  # noqa: F401
        import pybind11
        import sysconfig
    except ImportError:
        return None
    import jax

    lib = build(verbose=verbose)
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(OUT_DIR, "jax_finufft_gpu" + ext)
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    cmd = ["c++", "-O2", "-std=c++17", "-shared", "-fPIC",
           "-I", jax.ffi.include_dir(), "-I", pybind11.get_include(),
           "-I", sysconfig.get_paths()["include"], "-I", INCLUDE, "-I", cuda_inc,
           os.path.join(HERE, "xla", "gbn_xla_ffi.cc"), "-L", OUT_DIR, "-lgbnufft",
           "-Wl,-rpath," + OUT_DIR, "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("XLA FFI module build failed:\n%s%s" % (r.stdout, r.stderr))
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
