"""ctypes binding of libbemgpu.so (declared in include/bemgpu.h).

The library is built in-tree by bem_gb300/build.py.  There is no fallback:
if the library is missing or cannot be loaded, importing the compute API
raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbemgpu.so")

OK = 0
ERR_ARG, ERR_OOM, ERR_CUDA, ERR_SINGULAR, ERR_NO_CONVERGE, ERR_TIMEOUT, ERR_MESH = -1, -2, -3, -4, -5, -6, -7
ERR_CANCELLED = -8
PENDING = 1
K_NAMES = ["fill_far", "fill_near", "gather", "lu_panel", "lu_gemm", "trsm", "solve_gemm", "trace", "refine_gemm",
           "near_spmm", "slice"]
TUNE_NEAR_MINB, TUNE_FAR_ROWS, TUNE_RASTER, TUNE_PANEL_CTAS, TUNE_NEAR_SYNC, TUNE_NEAR_GRID, TUNE_EX_WIDE, \
    TUNE_LU_SUPER = range(8)
PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_LA = 2

ERR_NAMES = {ERR_ARG: "BEMGPU_ERR_ARG", ERR_OOM: "BEMGPU_ERR_OOM", ERR_CUDA: "BEMGPU_ERR_CUDA",
             ERR_SINGULAR: "BEMGPU_ERR_SINGULAR", ERR_NO_CONVERGE: "BEMGPU_ERR_NO_CONVERGE",
             ERR_TIMEOUT: "BEMGPU_ERR_TIMEOUT", ERR_MESH: "BEMGPU_ERR_MESH", ERR_CANCELLED: "BEMGPU_ERR_CANCELLED"}

# Every symbol include/bemgpu.h declares.
EXPORTED = [
    "bemgpu_ctx_create", "bemgpu_ctx_destroy", "bemgpu_ctx_last_error", "bemgpu_version",
    "bemgpu_ctx_stream", "bemgpu_ctx_launches", "bemgpu_ctx_set_engines", "bemgpu_prof_enable", "bemgpu_prof_query", "bemgpu_prof_query_tensor",
    "bemgpu_geom_create", "bemgpu_geom_destroy", "bemgpu_tree_create", "bemgpu_tree_destroy",
    "bemgpu_tree_size", "bemgpu_mesh_rwgs", "bemgpu_green_init", "bemgpu_options_default", "bemgpu_theta",
    "bemgpu_dimensionless_omega", "bemgpu_zts", "bemgpu_zts_host", "bemgpu_heat_transfer",
    "bemgpu_zts_noalloc", "bemgpu_cgemm", "bemgpu_cgemm_acc64", "bemgpu_zgemm_exact",
    "bemgpu_farm_create", "bemgpu_farm_destroy", "bemgpu_farm_lanes", "bemgpu_farm_lane_ctx", "bemgpu_farm_submit",
    "bemgpu_farm_poll", "bemgpu_farm_cancel", "bemgpu_farm_last_error", "bemgpu_farm_set_budget",
    "bemgpu_farm_budget", "bemgpu_ctx_workspace_bytes", "bemgpu_ctx_trim", "bemgpu_solve_footprint", "bemgpu_ctx_solve_footprint",
    "bemgpu_ctx_set_solver", "bemgpu_ctx_wait_selftest", "bemgpu_ctx_set_escalation_tol", "bemgpu_ctx_set_fp64_fallback_tol",
    "bemgpu_zgemm_exact_quantized", "bemgpu_tree_create_body_device", "bemgpu_tree_concat", "bemgpu_tree_rwgs",
    "bemgpu_ctx_set_tuning", "bemgpu_ctx_get_tuning", "bemgpu_heat_transfer_batch", "bemgpu_batch_footprint",
    "bemgpu_farm_set_batch", "bemgpu_pending_free_bytes",
]


class Green(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double * 2) for n in
                ("eps", "mu", "omega", "ksquared", "k", "ik", "k2", "Zeps", "Zmu")] + [("external", ctypes.c_int)]


class Options(ctypes.Structure):
    _fields_ = [("farThresh6", ctypes.c_double), ("farThresh10", ctypes.c_double),
                ("farThresh15", ctypes.c_double), ("farThresh21", ctypes.c_double)]


class SolveReq(ctypes.Structure):
    _fields_ = [("a", ctypes.c_double), ("eV", ctypes.c_double), ("T1", ctypes.c_double), ("T2", ctypes.c_double),
                ("eps1", ctypes.c_double * 2), ("mu1", ctypes.c_double * 2),
                ("eps2", ctypes.c_double * 2), ("mu2", ctypes.c_double * 2)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("ms_fill", ctypes.c_double), ("ms_lu", ctypes.c_double), ("ms_solve", ctypes.c_double),
                ("ms_trace", ctypes.c_double), ("ms_refine", ctypes.c_double),
                ("S_re", ctypes.c_double), ("S_im", ctypes.c_double), ("err_est", ctypes.c_double),
                ("refine_iters", ctypes.c_int),
                ("pairs_near", ctypes.c_int64), ("pairs_far_fp64", ctypes.c_int64), ("pairs_far_fp32", ctypes.c_int64),
                ("ms_queued", ctypes.c_double), ("ms_latency", ctypes.c_double), ("solver", ctypes.c_int)]


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libbemgpu.so; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    vp, i32, i64, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    P = ctypes.POINTER
    sig = {
        "bemgpu_ctx_create": (i32, [i32, P(vp)]),
        "bemgpu_ctx_destroy": (i32, [vp]),
        "bemgpu_ctx_last_error": (ctypes.c_char_p, [vp]),
        "bemgpu_version": (ctypes.c_char_p, []),
        "bemgpu_ctx_stream": (i32, [vp, P(vp)]),
        "bemgpu_ctx_launches": (i64, [vp]),
        "bemgpu_ctx_set_engines": (i32, [vp, i32, i32]),
        "bemgpu_prof_enable": (i32, [vp, i32]),
        "bemgpu_prof_query": (i32, [vp, i32, P(i64), P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double)]),
        "bemgpu_prof_query_tensor": (i32, [vp, i32, P(ctypes.c_double)]),
        "bemgpu_geom_create": (i32, [vp, dp, i32, dp, i32, P(vp)]),
        "bemgpu_geom_destroy": (i32, [vp]),
        "bemgpu_tree_create": (i32, [vp, dp, i32, P(vp)]),
        "bemgpu_tree_destroy": (i32, [vp]),
        "bemgpu_tree_size": (i32, [vp]),
        "bemgpu_tree_create_body_device": (i32, [vp, i32, i32, P(vp)]),
        "bemgpu_tree_concat": (i32, [vp, vp, P(vp)]),
        "bemgpu_tree_rwgs": (i32, [vp, dp, i32]),
        "bemgpu_mesh_rwgs": (i32, [dp, i32, i32, dp, i32, P(i32)]),
        "bemgpu_green_init": (i32, [dp, dp, dp, i32, P(Green)]),
        "bemgpu_options_default": (None, [P(Options)]),
        "bemgpu_theta": (ctypes.c_double, [ctypes.c_double, ctypes.c_double]),
        "bemgpu_dimensionless_omega": (ctypes.c_double, [ctypes.c_double, ctypes.c_double]),
        "bemgpu_zts": (i32, [vp, vp, vp, P(Green), P(Options), i32, vp, i64, vp]),
        "bemgpu_zts_host": (i32, [vp, vp, vp, P(Green), P(Options), i32, dp, i64]),
        "bemgpu_zts_noalloc": (i32, [vp, vp, vp, P(Green), P(Options), vp, i64, vp]),
        "bemgpu_cgemm": (i32, [vp, i32, i32, i32, vp, i64, vp, i64, vp, i64, i32, i32]),
        "bemgpu_cgemm_acc64": (i32, [vp, i32, i32, i32, vp, i64, vp, i64, vp, i64, i32, i32]),
        "bemgpu_zgemm_exact": (i32, [vp, i32, i32, i32, vp, i64, vp, i64, vp, i64, i32, i32]),
        "bemgpu_zgemm_exact_quantized": (i32, [vp, i32, i32, i32, vp, i64, vp, i64, vp, i64, i32]),
        "bemgpu_heat_transfer": (i32, [vp, vp, vp, vp, P(SolveReq), P(Options), i32, P(ctypes.c_double), P(SolveInfo)]),
        "bemgpu_heat_transfer_batch": (i32, [vp, i32, P(vp), P(vp), P(vp), P(SolveReq), P(Options), i32,
                                             P(ctypes.c_double), P(SolveInfo), P(i32)]),
        "bemgpu_batch_footprint": (i64, [i32, i32, i32, i32]),
        "bemgpu_farm_create": (i32, [i32, i32, P(vp)]),
        "bemgpu_farm_destroy": (i32, [vp]),
        "bemgpu_farm_lanes": (i32, [vp]),
        "bemgpu_farm_set_batch": (i32, [vp, i32]),
        "bemgpu_farm_lane_ctx": (i32, [vp, i32, P(vp)]),
        "bemgpu_farm_submit": (i32, [vp, vp, vp, vp, P(SolveReq), P(Options), i32, P(i64)]),
        "bemgpu_farm_poll": (i32, [vp, i64, ctypes.c_double, P(ctypes.c_double), P(SolveInfo)]),
        "bemgpu_farm_cancel": (i32, [vp, i64]),
        "bemgpu_farm_last_error": (ctypes.c_char_p, [vp]),
        "bemgpu_farm_set_budget": (i32, [vp, i64]),
        "bemgpu_farm_budget": (i64, [vp]),
        "bemgpu_ctx_workspace_bytes": (i64, [vp]),
        "bemgpu_ctx_trim": (i32, [vp]),
        "bemgpu_pending_free_bytes": (i64, []),
        "bemgpu_solve_footprint": (i64, [i32, i32, i32]),
        "bemgpu_ctx_solve_footprint": (i64, [vp, i32, i32, i32]),
        "bemgpu_ctx_set_solver": (i32, [vp, i32]),
        "bemgpu_ctx_set_tuning": (i32, [vp, i32, i32]),
        "bemgpu_ctx_get_tuning": (i32, [vp, i32, P(i32)]),
        "bemgpu_ctx_wait_selftest": (i32, [vp, i64]),
        "bemgpu_ctx_set_escalation_tol": (i32, [vp, ctypes.c_double]),
        "bemgpu_ctx_set_fp64_fallback_tol": (i32, [vp, ctypes.c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class BemGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code
