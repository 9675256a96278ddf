"""The FP32 fold's integer fast path against the FP64 chain, on the host.

jax-finufft_gb300/csrc/gbn_fold.cuh is host-compilable; this builds
tests/fold_fast_check.cpp against it with g++ and walks a stride of all 2^32
float bit patterns (hashed, so every exponent range is covered) for several
grid sizes and kernel widths, odd widths included.  Every accepted point must
give the FP64 chain's grid start and FP32 offset bit for bit; the FP64 chain
is the fold of the CPU restatement (oracle/nufft_oracle.c), which the GPU fold
tests pin.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("foldfast") / "fold_fast_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread",
                    "-I", os.path.join(ROOT, "jax-finufft_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "fold_fast_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("nf, w", [(512, 6), (540, 7), (1024, 8), (16, 2), (4096, 16),
                                   (270, 5), (100000, 13), (1 << 20, 6)])
def test_fold_fast_path_matches_fp64_chain(checker, nf, w):
    threads = max(1, min(8, os.cpu_count() or 1))
    out = subprocess.run([checker, str(nf), str(w), "97", str(threads)], check=True,
                         capture_output=True, text=True).stdout.split()
    accepted, mismatches = int(out[0]), int(out[1])
    assert mismatches == 0
    # most finite patterns in range are accepted (non-finite, zero, subnormal
    # and |x| >= 2^22 pi are always declined)
    assert accepted > (1 << 32) // 97 // 10


@pytest.mark.parametrize("nf, w", [(512, 6), (540, 7), (1024, 8), (128, 2), (4096, 16)])
def test_fold_fast_path_at_grid_boundaries(checker, nf, w):
    """Floats within 64 ulps of every grid cell and half cell."""
    out = subprocess.run([checker, str(nf), str(w), "1", "1", "boundary"], check=True,
                         capture_output=True, text=True).stdout.split()
    accepted, mismatches = int(out[0]), int(out[1])
    assert mismatches == 0
    assert accepted > 0
