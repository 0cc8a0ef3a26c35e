"""A small autotuner: time candidate launch configurations with CUDA events and keep the fastest.

Results are cached per problem signature for the life of the process, and optionally in a JSON
file (``FFMPM_TUNE_CACHE``) so a later process reuses them.
"""
from __future__ import annotations

import json
import os
from typing import Callable, Hashable, Sequence

import torch

_CACHE: dict = {}


def _file_cache_path():
    return os.environ.get("FFMPM_TUNE_CACHE")


def _load_file_cache():
    path = _file_cache_path()
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value):
    _CACHE[key] = value
    path = _file_cache_path()
    if path:
        data = _load_file_cache()
        data[key] = value
        with open(path, "w") as f:
            json.dump(data, f)


def time_call(fn: Callable[[], None], iters: int = 3, warmup: int = 1) -> float:
    """Average milliseconds of fn() on the current stream (CUDA events, synchronised)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / iters


def tune(signature: Hashable, candidates: Sequence, run: Callable[[object], None], iters: int = 3,
         warmup: int = 1) -> tuple:
    """Return (best candidate, {candidate: ms}); cached by signature."""
    key = json.dumps(signature, default=str)
    if key in _CACHE:
        return tuple(_CACHE[key]) if isinstance(_CACHE[key], list) else _CACHE[key], {}
    disk = _load_file_cache()
    if key in disk:
        best = disk[key]
        best = tuple(best) if isinstance(best, list) else best
        _CACHE[key] = best
        return best, {}
    timings = {}
    for c in candidates:
        try:
            timings[c] = time_call(lambda: run(c), iters=iters, warmup=warmup)
        except RuntimeError:
            continue  # a configuration that cannot launch here is skipped
    if not timings:
        raise RuntimeError("autotune: no candidate configuration ran")
    best = min(timings, key=timings.get)
    _store(key, list(best) if isinstance(best, tuple) else best)
    return best, timings
