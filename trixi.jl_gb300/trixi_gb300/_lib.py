"""ctypes binding of libtrixi_gb300.so (include/trixi_gb300.h).

The library is built in-tree (trixi.jl_gb300/_build).  There is no fallback:
if the shared library cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libtrixi_gb300.so")

TG_OK = 0
(TG_ERR_INVALID_ARGUMENT, TG_ERR_UNSUPPORTED, TG_ERR_CUDA, TG_ERR_NUMERICAL,
 TG_ERR_STATE) = -1, -2, -3, -4, -5
STATUS_NAMES = {-1: "invalid argument", -2: "unsupported", -3: "CUDA error",
                -4: "numerical failure", -5: "invalid call order"}

# enums (trixi_gb300.h)
TG_VOLUME_WEAK_FORM, TG_VOLUME_FLUX_DIFFERENCING, TG_VOLUME_SHOCK_CAPTURING_HG = 0, 1, 2
(TG_FLUX_CENTRAL, TG_FLUX_RANOCHA, TG_FLUX_SHIMA_ETAL, TG_FLUX_LAX_FRIEDRICHS,
 TG_FLUX_LAX_FRIEDRICHS_NAIVE, TG_FLUX_HLLC, TG_FLUX_CHANDRASHEKAR, TG_FLUX_HLLE) = range(8)
TG_SOURCE_NONE, TG_SOURCE_CONVERGENCE_TEST = 0, 1
TG_PRECISION_FP64, TG_PRECISION_MIXED = 0, 1
TG_MESH_TREE, TG_MESH_CURVED = 0, 1
TG_BOUNDARY_PERIODIC, TG_BOUNDARY_DIRICHLET, TG_BOUNDARY_SLIP_WALL = 0, 1, 2

# Every symbol declared in include/trixi_gb300.h.
EXPORTS = ("tg_api_version", "tg_ctx_create", "tg_ctx_destroy", "tg_last_error", "tg_ndofs",
           "tg_upload_state", "tg_download_state", "tg_prefetch_state", "tg_load_prefetched",
           "tg_fetch_state", "tg_transfer_wait", "tg_transfer_join", "tg_state_device_ptr", "tg_rhs",
           "tg_rhs_host", "tg_max_dt", "tg_rk_stage", "tg_rk_stage_part", "tg_step",
           "tg_step_enqueue", "tg_clock_read", "tg_set_time",
           "tg_integrals", "tg_alpha", "tg_status", "tg_synchronize",
           "tg_elements_per_block", "tg_stream", "tg_integrals_noalloc",
           "tg_vector_create", "tg_vector_destroy", "tg_vector_copy", "tg_lincomb", "tg_fma_peak", "tg_error_norms",
           "tg_mlp_create", "tg_mlp_destroy", "tg_mlp_nparams", "tg_mlp_get_params",
           "tg_mlp_set_params", "tg_mlp_harvest", "tg_mlp_dataset", "tg_mlp_train",
           "tg_mlp_gradient", "tg_mlp_predict", "tg_ctx_set_learned_indicator", "tg_mlp_last",
           "tg_entropy_timederivative", "tg_ensemble_create", "tg_ensemble_destroy",
           "tg_ensemble_size", "tg_ensemble_context", "tg_ensemble_step", "tg_ensemble_autotune",
           "tg_ensemble_threads_per_block", "tg_ensemble_last_error", "tg_ctx_autotune",
           "tg_amr_indicator", "tg_amr_indicator_max", "tg_adapt_state", "tg_tree_create", "tg_tree_destroy",
           "tg_tree_refine_patch", "tg_tree_nelements", "tg_tree_elements", "tg_tree_counts",
           "tg_tree_interfaces", "tg_tree_mortars", "tg_tree_adapt", "tg_tree_transfer_map")


class TrixiGB300Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{STATUS_NAMES.get(code, code)}] {msg}")
        self.code = code


class tg_config(ctypes.Structure):
    _fields_ = [
        ("ndims", ctypes.c_int32),
        ("polydeg", ctypes.c_int32),
        ("nelements", ctypes.c_int64),
        ("ninterfaces", ctypes.c_int64),
        ("gamma", ctypes.c_double),
        ("volume_integral", ctypes.c_int32),
        ("volume_flux", ctypes.c_int32),
        ("surface_flux", ctypes.c_int32),
        ("volume_flux_fv", ctypes.c_int32),
        ("alpha_max", ctypes.c_double),
        ("alpha_min", ctypes.c_double),
        ("alpha_smooth", ctypes.c_int32),
        ("source_terms", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("nodes", ctypes.POINTER(ctypes.c_double)),
        ("weights", ctypes.POINTER(ctypes.c_double)),
        ("inverse_weights", ctypes.POINTER(ctypes.c_double)),
        ("derivative_hat", ctypes.POINTER(ctypes.c_double)),
        ("derivative_split", ctypes.POINTER(ctypes.c_double)),
        ("inverse_vandermonde_legendre", ctypes.POINTER(ctypes.c_double)),
        ("neighbor_ids", ctypes.POINTER(ctypes.c_int64)),
        ("orientations", ctypes.POINTER(ctypes.c_int64)),
        ("inverse_jacobian", ctypes.POINTER(ctypes.c_double)),
        ("node_coordinates", ctypes.POINTER(ctypes.c_double)),
        ("elements_per_block", ctypes.c_int32),
        ("boundary_conditions", ctypes.c_int32 * 6),
        ("boundary_value_function", ctypes.c_int32),
        ("boundary_value_params", ctypes.c_double * 4),
        ("nmortars", ctypes.c_int64),
        ("mortar_neighbor_ids", ctypes.POINTER(ctypes.c_int64)),
        ("mortar_large_sides", ctypes.POINTER(ctypes.c_int64)),
        ("mortar_orientations", ctypes.POINTER(ctypes.c_int64)),
        ("mortar_forward_upper", ctypes.POINTER(ctypes.c_double)),
        ("mortar_forward_lower", ctypes.POINTER(ctypes.c_double)),
        ("mortar_reverse_upper", ctypes.POINTER(ctypes.c_double)),
        ("mortar_reverse_lower", ctypes.POINTER(ctypes.c_double)),
        ("mesh_type", ctypes.c_int32),
        ("contravariant_vectors", ctypes.POINTER(ctypes.c_double)),
    ]


_lib = None


def load(path: str | None = None):
    """Load the shared library (raises OSError if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"libtrixi_gb300.so not found at {path}: run trixi.jl_gb300/build.py "
                      "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    d, i32, i64, vp = ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    pd = P(d)
    sigs = {
        "tg_api_version": ([], ctypes.c_int),
        "tg_ctx_create": ([P(tg_config), P(vp)], ctypes.c_int),
        "tg_ctx_destroy": ([vp], ctypes.c_int),
        "tg_last_error": ([vp, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
        "tg_ndofs": ([vp, P(i64), P(i64)], ctypes.c_int),
        "tg_upload_state": ([vp, vp], ctypes.c_int),
        "tg_download_state": ([vp, vp], ctypes.c_int),
        "tg_prefetch_state": ([vp, ctypes.c_int32, vp], ctypes.c_int),
        "tg_load_prefetched": ([vp, ctypes.c_int32], ctypes.c_int),
        "tg_fetch_state": ([vp, ctypes.c_int32, vp], ctypes.c_int),
        "tg_transfer_wait": ([vp, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "tg_transfer_join": ([vp], ctypes.c_int),
        "tg_state_device_ptr": ([vp, P(vp)], ctypes.c_int),
        "tg_rhs": ([vp, vp, vp, d], ctypes.c_int),
        "tg_rhs_host": ([vp, vp, vp, d], ctypes.c_int),
        "tg_max_dt": ([vp, vp, pd], ctypes.c_int),
        "tg_rk_stage": ([vp, i32, d, d], ctypes.c_int),
        "tg_rk_stage_part": ([vp, i32, d, d, i32], ctypes.c_int),
        "tg_step": ([vp, i64, d, d, pd, P(i64)], ctypes.c_int),
        "tg_step_enqueue": ([vp, i64, d, d, d], ctypes.c_int),
        "tg_clock_read": ([vp, pd, P(i64), P(ctypes.c_int32)], ctypes.c_int),
        "tg_set_time": ([vp, d], ctypes.c_int),
        "tg_integrals": ([vp, pd], ctypes.c_int),
        "tg_alpha": ([vp, vp, pd], ctypes.c_int),
        "tg_amr_indicator": ([vp, ctypes.c_double, ctypes.c_double, i32, i32, pd], ctypes.c_int),
        "tg_amr_indicator_max": ([vp, i32, pd], ctypes.c_int),
        "tg_tree_create": ([i32, i32, pd, pd, P(i32), P(vp)], ctypes.c_int),
        "tg_tree_destroy": ([vp], ctypes.c_int),
        "tg_tree_refine_patch": ([vp, i32, pd, pd, d], ctypes.c_int),
        "tg_tree_nelements": ([vp, P(i64)], ctypes.c_int),
        "tg_tree_elements": ([vp, P(i32), pd], ctypes.c_int),
        "tg_tree_counts": ([vp, P(i64), P(i64)], ctypes.c_int),
        "tg_tree_interfaces": ([vp, P(i64), P(i64)], ctypes.c_int),
        "tg_tree_mortars": ([vp, P(i64), P(i64), P(i64)], ctypes.c_int),
        "tg_tree_adapt": ([vp, P(ctypes.c_int8), i32, i32, P(i32)], ctypes.c_int),
        "tg_tree_transfer_map": ([vp, P(i64), P(ctypes.c_int8)], ctypes.c_int),
        "tg_adapt_state": ([vp, vp, P(ctypes.c_int64), P(ctypes.c_int8), pd, pd, pd, pd],
                           ctypes.c_int),
        "tg_status": ([vp, P(i32)], ctypes.c_int),
        "tg_synchronize": ([vp], ctypes.c_int),
        "tg_elements_per_block": ([vp, P(i32)], ctypes.c_int),
        "tg_stream": ([vp, P(vp)], ctypes.c_int),
        "tg_vector_create": ([vp, i64, P(vp)], ctypes.c_int),
        "tg_vector_destroy": ([vp, vp], ctypes.c_int),
        "tg_vector_copy": ([vp, vp, vp, i64, i32], ctypes.c_int),
        "tg_lincomb": ([vp, i64, vp, d, vp, d, vp], ctypes.c_int),
        "tg_fma_peak": ([i32, pd], ctypes.c_int),
        "tg_error_norms": ([vp, vp, d, i32, pd, i32, pd, pd, pd, pd], ctypes.c_int),
        "tg_integrals_noalloc": ([i32, i32, i64, d, pd, vp, vp, vp, vp], ctypes.c_int),
        "tg_mlp_create": ([i32, i32, i32, ctypes.c_uint64, P(vp)], ctypes.c_int),
        "tg_mlp_destroy": ([vp], ctypes.c_int),
        "tg_mlp_nparams": ([vp, P(i64)], ctypes.c_int),
        "tg_mlp_get_params": ([vp, vp], ctypes.c_int),
        "tg_mlp_set_params": ([vp, vp], ctypes.c_int),
        "tg_mlp_harvest": ([vp, vp, i32, i32, P(i64)], ctypes.c_int),
        "tg_mlp_dataset": ([vp, vp, vp], ctypes.c_int),
        "tg_mlp_train": ([vp, i64, i32, ctypes.c_float, i32, ctypes.c_uint64,
                          P(ctypes.c_float)], ctypes.c_int),
        "tg_mlp_gradient": ([vp, vp, vp, i32, vp, P(ctypes.c_float)], ctypes.c_int),
        "tg_mlp_predict": ([vp, vp, i64, vp], ctypes.c_int),
        "tg_ctx_set_learned_indicator": ([vp, vp, ctypes.c_float], ctypes.c_int),
        "tg_mlp_last": ([vp, vp, vp, vp, vp], ctypes.c_int),
        "tg_entropy_timederivative": ([vp, d, pd], ctypes.c_int),
        "tg_ensemble_create": ([P(tg_config), i32, i32, P(vp)], ctypes.c_int),
        "tg_ensemble_destroy": ([vp], ctypes.c_int),
        "tg_ensemble_size": ([vp], ctypes.c_int),
        "tg_ensemble_context": ([vp, i32, P(vp)], ctypes.c_int),
        "tg_ensemble_step": ([vp, i64, d, d, pd, P(i64)], ctypes.c_int),
        "tg_ensemble_autotune": ([vp, i32, P(i32), pd], ctypes.c_int),
        "tg_ensemble_threads_per_block": ([vp], ctypes.c_int),
        "tg_ensemble_last_error": ([vp, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
        "tg_ctx_autotune": ([vp, i32, P(i32), pd], ctypes.c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def last_error(ctx=None) -> str:
    buf = ctypes.create_string_buffer(1024)
    load().tg_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, ctx=None) -> None:
    if rc != TG_OK:
        raise TrixiGB300Error(rc, last_error(ctx))
