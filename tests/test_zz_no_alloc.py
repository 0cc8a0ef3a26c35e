"""The allocation-free block sort, ffmpm_sort_by_block_static, called through the C ABI.

Some callers cannot allocate device memory (a host program that owns every GPU allocation and
passes plugins device pointers only, or a real-time loop that allows no allocation after
start-up).  For them the library offers a variant of the block sort whose scratch is a fixed
static array inside the library instead of a caller workspace.  Its output must equal the
workspace sort's bit for bit (integer keys and an index permutation), call after call, even
though every call reuses the same array, and its status word (handed over through the optional
status_out argument) must report out-of-grid particles for the call that had them only.
"""
import ctypes

import numpy as np
import pytest
import torch

from femflow_gb300 import _native as N
from femflow_gb300 import engine as E

pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sort_both(x: np.ndarray, res: int, det: bool):
    n, dim = x.shape
    prm = E.make_params(dim, res, torch.float32, 1 / res, float(res), 1e-4, deterministic=det)
    xd = torch.from_numpy(x).cuda()
    out = {}
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    for name in ("ws", "static"):
        keys = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        perm = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        if name == "ws":
            ws = E.Workspace(prm, n, "cuda")
            N.call("ffmpm_sort_by_block", ctypes.byref(prm), ctypes.c_void_p(xd.data_ptr()), n,
                   ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(ws.ptr),
                   ctypes.c_size_t(ws.bytes), _stream())
        else:
            N.call("ffmpm_sort_by_block_static", ctypes.byref(prm), ctypes.c_void_p(xd.data_ptr()), n,
                   ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(perm.data_ptr()),
                   ctypes.c_void_p(status.data_ptr()), _stream())
        torch.cuda.synchronize()
        out[name] = (keys.cpu().numpy(), perm.cpu().numpy())
    out["status"] = int(status.item())
    return out


@pytest.mark.parametrize("dim,res,det", [(3, 128, False), (2, 256, True)])
def test_static_sort_equals_workspace_sort_on_consecutive_calls(dim, res, det):
    rng = np.random.default_rng(11)
    # calls in a row with different inputs: each must see none of the previous one's leftovers,
    # neither in the keys and permutation nor in the status word
    for n, outside in ((N.STATIC_SORT_MAX_N, True), (100_003, False), (77_777, True)):
        x = rng.uniform(0.05, 0.95, size=(n, dim)).astype(np.float32)
        if outside:
            x[::1013] = 1.7  # outside the grid: sorted last with key 0xFFFFFFFF
        out = _sort_both(x, res, det)
        k_ws, p_ws = out["ws"]
        k_st, p_st = out["static"]
        assert np.array_equal(k_st, k_ws)
        assert np.array_equal(p_st, p_ws)
        assert np.array_equal(np.sort(p_st), np.arange(n))
        assert out["status"] == (N.STATUS_OOB if outside else 0), out["status"]


def test_static_sort_rejects_more_than_its_capacity():
    n = N.STATIC_SORT_MAX_N + 1
    prm = E.make_params(3, 64, torch.float32, 1 / 64, 64.0, 1e-4)
    x = torch.zeros((4, 3), device="cuda")
    rc = N.load().ffmpm_sort_by_block_static(ctypes.byref(prm), ctypes.c_void_p(x.data_ptr()), n, None, None,
                                             None, _stream())
    assert rc == N.ERR_CAPACITY
