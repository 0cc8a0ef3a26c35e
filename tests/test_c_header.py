"""The C ABI from C: include/femflow_mpm.h compiles as C11 (gcc, warnings as errors), a C program
links the built library, and host-only calls (workspace size, plan description) answer as they
do through the Python binding; the parameter struct has the size the library asserts (no GPU)."""
import ctypes
import os
import shutil
import subprocess

import pytest
import torch

from femflow_gb300 import _native as N
from femflow_gb300 import engine as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "femflow_mpm.h"
int main(void) {
  ffmpm_params p = {.dim = 3, .res = 128, .real_bytes = 4, .model = FFMPM_MODEL_NEO_HOOKEAN,
                    .dx = 1.0 / 128, .inv_dx = 128, .dt = 5e-5, .gravity = -9.8, .volume = 1e-6,
                    .hardening = 1.0};
  size_t bytes = 0;
  int64_t info[8] = {0};
  const int rc = ffmpm_workspace_size(&p, 1 << 20, &bytes);
  const int rc2 = ffmpm_plan_info(&p, 1 << 20, info);
  const int bad = ffmpm_workspace_size(NULL, 1 << 20, &bytes) == FFMPM_OK;
  printf("%d %d %d %zu %zu %lld %lld\n", rc, rc2, bad, sizeof(ffmpm_params), bytes, (long long)info[2],
         (long long)info[4]);
  return 0;
}
"""


def test_header_compiles_as_c_and_links(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc or not os.path.exists(N.LIB_PATH):
        pytest.skip("gcc or the built library not available")
    src = tmp_path / "abi.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "abi"
    libdir = os.path.dirname(N.LIB_PATH)
    libname = os.path.basename(N.LIB_PATH)[3:-3]  # lib<name>.so
    subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", libdir, f"-l{libname}", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                   check=True, capture_output=True, timeout=120)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    rc, rc2, bad, size, nbytes, blocks, passes = (int(t) for t in out.stdout.split())
    assert (rc, rc2, bad) == (N.OK, N.OK, 0)
    assert size == ctypes.sizeof(N.Params)
    # the same answers through the Python binding
    prm = E.make_params(3, 128, torch.float32, 1 / 128, 128.0, 5e-5, -9.8, 1e-6, 1.0)
    want = ctypes.c_size_t(0)
    N.call("ffmpm_workspace_size", ctypes.byref(prm), 1 << 20, ctypes.byref(want))
    assert nbytes == want.value
    info = (ctypes.c_int64 * 8)()
    N.call("ffmpm_plan_info", ctypes.byref(prm), 1 << 20, info)
    assert (blocks, passes) == (info[2], info[4]) == (17 ** 3, 3)
