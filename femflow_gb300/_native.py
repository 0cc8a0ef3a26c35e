"""ctypes binding of libfemflow_mpm.so (the sm_103a kernels behind include/femflow_mpm.h).

There is no CPU fallback: if the library is missing or no CUDA device is visible, every compute
call raises.  ``load()`` returns the library; ``call()`` raises ``RuntimeError`` on a non-zero
return code.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfemflow_mpm.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "femflow_mpm.h")

OK = 0
ERR_BADARG = 3
ERR_WORKSPACE = 4
ERR_CUDA = 5
ERR_UNSUPPORTED = 7
ERR_CAPACITY = 8
ERRORS = {ERR_BADARG: "bad argument", ERR_WORKSPACE: "workspace too small or misaligned", ERR_CUDA: "CUDA error",
          ERR_UNSUPPORTED: "unsupported configuration", ERR_CAPACITY: "more particles than the static scratch holds"}
STATIC_SORT_MAX_N = 262144

STATUS_OOB = 1
STATUS_NONFINITE = 2
STATUS_TIMEOUT = 4

INJECT_LOOKBACK_STALL = 1
INJECT_BARRIER_ABSENT = 2

MODELS = {"neo_hookean": 0, "snow": 1, "fixed_corotated": 2}
NPHASES = 7
PHASES = ("keys", "sort", "plan", "p2g", "grid_update", "g2p", "g2p2g")
WALLS = {"reference": 0, "sticky3": 1}


class Params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("res", ctypes.c_int32), ("real_bytes", ctypes.c_int32), ("model", ctypes.c_int32),
        ("wall_mode", ctypes.c_int32), ("deterministic", ctypes.c_int32), ("block_size", ctypes.c_int32),
        ("variant", ctypes.c_int32),
        ("dx", ctypes.c_double), ("inv_dx", ctypes.c_double), ("dt", ctypes.c_double), ("gravity", ctypes.c_double),
        ("volume", ctypes.c_double), ("hardening", ctypes.c_double), ("mass", ctypes.c_double),
        ("mu_0", ctypes.c_double), ("lambda_0", ctypes.c_double),
        ("n_planes", ctypes.c_int32), ("plane_rule", ctypes.c_int32), ("planes", (ctypes.c_double * 6) * 8),
        ("wait_limit", ctypes.c_uint32), ("inject", ctypes.c_uint32),
    ]


MAX_PLANES = 8
PLANE_RULES = {"sticky": 0, "reference_literal": 1}


class Particles(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("x", ctypes.c_void_p), ("v", ctypes.c_void_p), ("F", ctypes.c_void_p),
                ("C", ctypes.c_void_p), ("Jp", ctypes.c_void_p), ("mass", ctypes.c_void_p), ("mu_0", ctypes.c_void_p),
                ("lambda_0", ctypes.c_void_p), ("stride", ctypes.c_int64)]


class Grid(ctypes.Structure):
    _fields_ = [("velocity", ctypes.c_void_p), ("mass", ctypes.c_void_p)]


class Adjoint(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("v", ctypes.c_void_p), ("F", ctypes.c_void_p), ("C", ctypes.c_void_p),
                ("mu_0", ctypes.c_void_p), ("lambda_0", ctypes.c_void_p)]


MLP_IN, MLP_FEATURES, MLP_HIDDEN, MLP_OUT, MLP_PARAMS = 128, 113, 64, 12, 41168
MLP_OFF = {"W1": 0, "W2": 16384, "W3": 24576, "W4": 32768, "b1": 40960, "b2": 41024, "b3": 41088, "b4": 41152}


class MLP(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("W1", "W2", "W3", "W4", "b1", "b2", "b3", "b4", "in_scale",
                                                "out_scale")]


class MLPTrainer(ctypes.Structure):
    _fields_ = [("max_batch", ctypes.c_int32)] + [(k, ctypes.c_void_p) for k in (
        "params", "grads", "adam_m", "adam_v", "W1", "W2", "W3", "W4", "W2t", "W3t", "W4t", "Z1", "Z2", "Z3", "Y",
        "dH", "H1", "H2", "H3", "H1t", "H2t", "H3t", "Xt", "dY", "dZ", "dYt", "dZt", "status")]


_lib = None
_lock = threading.Lock()

_P = ctypes.POINTER
_vp = ctypes.c_void_p
_PROTOS = {
    "ffmpm_workspace_size": (ctypes.c_int, [_P(Params), ctypes.c_int64, _P(ctypes.c_size_t)]),
    "ffmpm_workspace_init": (ctypes.c_int, [_P(Params), ctypes.c_int64, _vp, ctypes.c_size_t, _vp]),
    "ffmpm_status_read": (ctypes.c_int, [_vp, _P(ctypes.c_int32), _P(ctypes.c_uint32), _vp]),
    "ffmpm_status_clear": (ctypes.c_int, [_vp, _vp]),
    "ffmpm_p2g": (ctypes.c_int, [_P(Params), _P(Particles), _P(Grid), _vp, ctypes.c_size_t, _vp]),
    "ffmpm_grid_op": (ctypes.c_int, [_P(Params), _P(Grid), _vp]),
    "ffmpm_g2p": (ctypes.c_int, [_P(Params), _P(Grid), _P(Particles), _vp, ctypes.c_size_t, _vp]),
    "ffmpm_substep": (ctypes.c_int, [_P(Params), _P(Particles), _vp, ctypes.c_size_t, _vp]),
    "ffmpm_substep_host": (ctypes.c_int, [_P(Params), _P(Particles), _P(Particles), _vp, ctypes.c_size_t, _vp]),
    "ffmpm_substeps_sorted": (ctypes.c_int, [_P(Params), _P(Particles), _P(Particles), _vp, _vp, ctypes.c_int32,
                                             _vp, ctypes.c_size_t, _vp]),
    "ffmpm_substeps_sorted_snapshots": (ctypes.c_int, [_P(Params), _P(Particles), _P(Particles), _vp, _vp,
                                                       ctypes.c_int32, _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "ffmpm_sort_by_block": (ctypes.c_int, [_P(Params), _vp, ctypes.c_int64, _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "ffmpm_diagnostics_fp64": (ctypes.c_int, [_P(Params), _P(Particles), _vp, _vp]),
    "ffmpm_profile_substeps": (ctypes.c_int, [_P(Params), _P(Particles), _P(Particles), _vp, _vp, ctypes.c_int32,
                                              _vp, ctypes.c_size_t, _vp, _P(ctypes.c_double), _P(ctypes.c_int64)]),
    "ffmpm_check_collision_points": (ctypes.c_int, [_P(Params), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                     ctypes.c_void_p, ctypes.c_void_p]),
    "ffmpm_plan_info": (ctypes.c_int, [_P(Params), ctypes.c_int64, _P(ctypes.c_int64)]),
    "ffmpm_kernels_per_call": (ctypes.c_int, [_P(Params), ctypes.c_int64, ctypes.c_int32, _P(ctypes.c_int64)]),
    "ffmpm_sort_by_block_static": (ctypes.c_int, [_P(Params), _vp, ctypes.c_int64, _vp, _vp, _vp, _vp]),
    "ffmpm_batch2d_workspace_size": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32, _P(ctypes.c_size_t)]),
    "ffmpm_batch2d_init": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_size_t, _vp]),
    "ffmpm_batch2d_substeps": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _P(Particles), ctypes.c_int32,
                                              ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_size_t, _vp]),
    "ffmpm_batch2d_status": (ctypes.c_int, [_vp, _P(ctypes.c_int32), _vp]),
    "ffmpm_batch2d_set_waits": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, _vp]),
    "ffmpm_adjoint_workspace_size": (ctypes.c_int, [_P(Params), ctypes.c_int64, _P(ctypes.c_size_t)]),
    "ffmpm_substep_adjoint": (ctypes.c_int, [_P(Params), _P(Particles), _P(Adjoint), _vp, ctypes.c_size_t, _vp]),
    "ffmpm_tc_gemm_bf16": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32, _vp, _vp]),
    "ffmpm_corrector_g2p": (ctypes.c_int, [_P(Params), _P(Grid), _P(Particles), _vp, _vp, _vp, _vp, _vp]),
    "ffmpm_mlp_train_forward": (ctypes.c_int, [_P(MLPTrainer), _vp, ctypes.c_int32, _vp]),
    "ffmpm_mlp_train_backward": (ctypes.c_int, [_P(MLPTrainer), _vp, _vp, ctypes.c_int32, _vp, _vp]),
    "ffmpm_mlp_train_update": (ctypes.c_int, [_P(MLPTrainer), ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_int32, _vp]),
    "ffmpm_implicit_points_workspace_size": (ctypes.c_int, [ctypes.c_int32, _P(ctypes.c_size_t)]),
    "ffmpm_implicit_points": (ctypes.c_int, [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_int32, _vp,
                                             ctypes.c_int64, _vp, _vp, ctypes.c_size_t, _vp]),
    "ffmpm_version": (ctypes.c_char_p, []),
}


def header_symbols() -> list[str]:
    """Names of every function declared in include/femflow_mpm.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(ffmpm_\w+)\s*\(", text, flags=re.M)))


def load(build_if_missing: bool = False):
    """Load the shared library (building it first when asked and the toolkit is present)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if build_if_missing:
                from . import build as _build

                _build.build()
            else:
                raise ImportError(
                    f"femflow_gb300 native library not built ({LIB_PATH}); run "
                    "`python -c 'import __graft_entry__ as g; g.build()'` first. There is no CPU fallback.")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name: str, *args) -> None:
    rc = getattr(load(), name)(*args)
    if rc != OK:
        raise RuntimeError(f"{name} failed: {ERRORS.get(rc, rc)}")
