"""The voxelizer's counter-block decode, shared by the device, host-buffer
and no-allocation generation entry points: a binning overflow flagged by the
device must come back as an error from every one of them, not as a
successful call with damaged output.  Checked on the CPU by a host build of
the decode (tests/native/tissue_status_check.cu)."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "tissue_status_check.cu")


def test_overflow_status_is_an_error(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "status_check")
    subprocess.run([nvcc, "-O1", "-std=c++17", "-Xcompiler", "-fopenmp", "-I",
                    os.path.join(ROOT, "include"), SRC, "-o", exe, "-lgomp"],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
