"""The 2D reference walls as node-index bounds (wall_band_2d in csrc/mpm_kernels.cuh) select exactly
the nodes that two_d/grid_op.py:13-19 selects with its float64 comparisons of i / res against 0.05
and 1 - 0.05, for every grid resolution up to 16,384 (CPU: the host function compiled by nvcc)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "mpm_kernels.cuh"
int main() {
  long bad = 0;
  for (int res = 1; res <= 16384; ++res) {
    int lo = 0, hi = 0;
    ffmpm::wall_band_2d(res, &lo, &hi);
    for (int i = 0; i <= res; ++i) {
      const double x = double(i) / double(res);
      if ((i < lo) != (x < 0.05) || (i > hi) != (x > 1.0 - 0.05)) ++bad;
    }
  }
  std::printf("%ld\n", bad);
  return bad != 0;
}
"""


def test_wall_band_bounds_equal_the_reference_comparisons(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "wall_band.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "wall_band"
    cmd = [nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "femflow_gb300", "csrc"),
           str(src), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, timeout=300)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "0", out.stdout + out.stderr
