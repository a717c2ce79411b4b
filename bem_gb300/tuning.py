"""Autotuner of the hot path's launch shapes.

The library exposes its launch-shape knobs per context (bemgpu_ctx_set_tuning,
include/bemgpu.h): the register budget of the double-float near-pair kernel
(CTAs per SM), the far-pair kernel's warps per CTA, and the rasterization band
of the tensor-core products.  None changes a result; each changes how fast
one kernel class runs on a given workload.  tune() times every candidate
value of each knob on the caller's own solve with the library's CUDA-event
kernel statistics (bemgpu_prof_*, summed over the kernel classes the knob
touches), keeping the others at their best so far (coordinate descent), and
returns the fastest settings.  Results are cached per GPU and size class (the
number of unknowns rounded to a power of two) in a JSON file, so a serving
process tunes each class once: $BEM_GB300_TUNING, else
~/.cache/bem_gb300/tuning.json.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import threading

from . import _lib

# knob name -> (library id, candidates, kernel classes whose time it sets)
KNOBS = {
    "near_minb": (_lib.TUNE_NEAR_MINB, (2, 3, 4), ("fill_near",)),
    "far_rows": (_lib.TUNE_FAR_ROWS, (1, 2, 4, 8), ("fill_far",)),
    "raster": (_lib.TUNE_RASTER, (4, 8, 16), ("lu_gemm", "trsm", "solve_gemm", "trace", "refine_gemm")),
}
DEFAULTS = {"near_minb": 2, "far_rows": 4, "raster": 8}

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("BEM_GB300_TUNING") or os.path.join(os.path.expanduser("~"), ".cache", "bem_gb300",
                                                               "tuning.json")


def size_class(n_unknowns: int) -> str:
    """Power-of-two bucket of the number of unknowns (N = 2 (Ns + Nt))."""
    return f"n{2 ** max(0, math.ceil(math.log2(max(1, n_unknowns))))}"


def gpu_name(device: int = 0) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda"


def apply(ctx_handle, params: dict) -> None:
    """Sets every knob of ``params`` on a context (a bemgpu_ctx_t handle)."""
    L = _lib.load()
    for name, value in params.items():
        knob = KNOBS[name][0]
        rc = L.bemgpu_ctx_set_tuning(ctx_handle, knob, int(value))
        if rc != _lib.OK:
            raise _lib.BemGpuError(rc, L.bemgpu_ctx_last_error(ctx_handle).decode())


def current(ctx_handle) -> dict:
    L = _lib.load()
    out = {}
    for name, (knob, _, _) in KNOBS.items():
        v = ctypes.c_int()
        L.bemgpu_ctx_get_tuning(ctx_handle, knob, ctypes.byref(v))
        out[name] = v.value
    return out


def _class_ms(ctx_handle, kinds) -> float:
    L = _lib.load()
    tot = 0.0
    for name in kinds:
        k = _lib.K_NAMES.index(name)
        n = ctypes.c_int64()
        ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        L.bemgpu_prof_query(ctx_handle, k, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(by))
        tot += ms.value
    return tot


def tune(solve, ctx_handle, reps: int = 2) -> tuple[dict, dict]:
    """Coordinate descent over KNOBS on one workload.  ``solve()`` runs one
    solve of the caller's workload on the context ``ctx_handle``.  Returns
    (best settings, {knob: {candidate: ms}}) and leaves the best applied."""
    L = _lib.load()
    best = dict(DEFAULTS)
    apply(ctx_handle, best)
    solve()  # workspace and module loading outside the measurement
    timings = {}
    for name, (_, cands, kinds) in KNOBS.items():
        timings[name] = {}
        for v in cands:
            apply(ctx_handle, dict(best, **{name: v}))
            solve()
            L.bemgpu_prof_enable(ctx_handle, 1)
            for _ in range(reps):
                solve()
            timings[name][v] = _class_ms(ctx_handle, kinds) / reps
            L.bemgpu_prof_enable(ctx_handle, 0)
        best[name] = min(timings[name], key=timings[name].get)
        apply(ctx_handle, best)
    return best, timings


def load_cache(path: str | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def store(key: str, params: dict, path: str | None = None) -> None:
    path = path or cache_path()
    with _lock:
        data = load_cache(path)
        data[key] = params
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def cache_key(n_unknowns: int, device: int = 0) -> str:
    return f"{gpu_name(device)}|{size_class(n_unknowns)}"


def tuned(solve, ctx_handle, n_unknowns: int, device: int = 0, path: str | None = None, retune: bool = False):
    """The cached settings of this GPU and size class, tuning (and caching)
    them on ``solve`` first when there are none.  Returns (settings, source)
    with source "cache" or "tuned"; the settings are applied to ctx_handle."""
    key = cache_key(n_unknowns, device)
    if not retune:
        hit = load_cache(path).get(key)
        if hit and set(hit) >= set(KNOBS):
            params = {k: hit[k] for k in KNOBS}
            apply(ctx_handle, params)
            return params, "cache"
    params, _ = tune(solve, ctx_handle)
    store(key, params, path)
    return params, "tuned"
