"""Compile the C restatement (nufft_oracle.c) into oracle/_build.

Test infrastructure only.  Run directly (``python -m oracle.build``) or through
``__graft_entry__.build()``.  gcc with OpenMP; -ffp-contract=off keeps one
rounding per double operation so folds and bins match the CUDA kernels bit for
bit.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nufft_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")


def library_path():
    return os.path.join(OUT_DIR, "libnufft_oracle.so")


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    out = library_path()
    tmp = out + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11",
           "-shared", "-fPIC", SRC, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
