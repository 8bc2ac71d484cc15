"""GPU checks of the device arithmetic helpers that replace plain float
operations on the hot path (asg_common.cuh): the packed f32x2 distances
(norm2_rn_x2, bit-identical to norm2_rn) and the cell-edge division by the box
side from a rounded reciprocal (div_rn_by, bit-identical to IEEE division).
tests/gpu_checks/helpers_check.cu is compiled for sm_103a here and run once."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_arithmetic_helpers_match_plain_operations(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "helpers_check"
    src = os.path.join(HERE, "gpu_checks", "helpers_check.cu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-o", str(exe), src], check=True, capture_output=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 5, r.stdout + r.stderr
    assert all("mismatches 0" in ln and "no error" in ln for ln in lines), r.stdout
    assert r.returncode == 0
