"""The voxelizer's two-float fast path never changes a result: on the CPU
(host build of the same __host__ __device__ evaluation code) every candidate
it decides must equal the FP64 replay of the reference arithmetic, for
random fibers and for lattice-aligned fibers that produce exact ties."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "voxel_fastpath_check.cu")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("vcheck") / "vcheck")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-fmad=false", "-Xcompiler",
                    "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe],
                   check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("seed,n,mode", [(11, 120, 0), (12, 120, 1), (13, 60, 0)])
def test_fast_path_matches_fp64(checker, seed, n, mode):
    r = subprocess.run([checker, str(seed), str(n), str(mode)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = r.stdout.split()
    frac = float(fields[4].strip("()"))
    assert frac > (0.95 if mode else 0.999), r.stdout
