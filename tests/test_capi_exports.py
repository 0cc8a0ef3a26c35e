"""The C-ABI library loads and exports every symbol declared in include/femflow_mpm.h (CPU only).

Only host-side entry points that launch nothing are called here.
"""
import ctypes
import os

import pytest

from femflow_gb300 import _native as N


def _lib():
    if not os.path.exists(N.LIB_PATH):
        pytest.skip("library not built")
    return N.load()


def test_header_symbols_parsed():
    syms = N.header_symbols()
    for s in ("ffmpm_substep", "ffmpm_p2g", "ffmpm_grid_op", "ffmpm_g2p", "ffmpm_substeps_sorted",
              "ffmpm_sort_by_block", "ffmpm_diagnostics_fp64", "ffmpm_workspace_size"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    lib = _lib()
    missing = [s for s in N.header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_string():
    assert b"sm_103a" in _lib().ffmpm_version()


def _params(**kw):
    from femflow_gb300 import engine as E
    import torch
    d = dict(dim=3, res=128, dtype=torch.float32, dx=1 / 128, inv_dx=128.0, dt=5e-5)
    d.update(kw)
    return E.make_params(**d)


def test_workspace_size_host_only():
    _lib()
    from femflow_gb300 import engine as E
    b1 = E.workspace_bytes(_params(), 1 << 20)
    b2 = E.workspace_bytes(_params(), 1 << 10)
    assert b1 > b2 > 0
    # two dense float4 grids of 129^3 nodes dominate at small n
    assert b2 > 2 * 129 ** 3 * 16
    # float64 grids are twice as large
    import torch
    assert E.workspace_bytes(_params(dtype=torch.float64), 1 << 10) > 2 * 129 ** 3 * 32


@pytest.mark.parametrize("bad", [dict(dim=4), dict(res=1), dict(block_size=3), dict(block_size=32)])
def test_workspace_size_rejects_bad_params(bad):
    _lib()
    from femflow_gb300 import engine as E
    p = _params()
    for k, v in bad.items():
        setattr(p, k, v)
    out = ctypes.c_size_t(0)
    rc = N.load().ffmpm_workspace_size(ctypes.byref(p), 100, ctypes.byref(out))
    assert rc == N.ERR_BADARG


def test_workspace_size_rejects_negative_n():
    _lib()
    out = ctypes.c_size_t(0)
    assert N.load().ffmpm_workspace_size(ctypes.byref(_params()), -1, ctypes.byref(out)) == N.ERR_BADARG
