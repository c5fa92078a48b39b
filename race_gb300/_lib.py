"""ctypes binding of the engine's C ABI (include/race_gb300.h).

The shared library is the in-tree build race_gb300/_build/librace_gb300.so.
Loading fails loudly when it is missing: there is no CPU implementation of
the engine.
"""
from __future__ import annotations

import ctypes as C
import pathlib

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "librace_gb300.so"

RACE_SUCCESS = 0
RACE_ERR_INVALID_ARG = 1
RACE_ERR_GRAPH_TRAVERSAL = 5
RACE_ERR_INCOMPATIBILITY = 6
ERRORS = {
    0: "RACE_SUCCESS", 1: "RACE_ERR_INVALID_ARG", 2: "RACE_ERR_MATRIX_SYMM", 3: "RACE_ERR_D2_COLOR",
    4: "RACE_ERR_D1_COLOR", 5: "RACE_ERR_GRAPH_TRAVERSAL", 6: "RACE_ERR_INCOMPATIBILITY", 7: "RACE_ERR_HWLOC",
    8: "RACE_ERR_PIN", 9: "RACE_ERR_INTERNAL", 10: "RACE_ERR_NOT_IMPLEMENTED", 100: "RACE_ERR_CUDA",
    101: "RACE_ERR_TIMEOUT",
}

# Symbols declared in include/race_gb300.h (checked by the CPU test suite).
EXPORTS = [
    "race_params_from_env", "race_create", "race_destroy", "race_set_stream", "race_color", "race_power_prepare",
    "race_get_perm", "race_get_num_threads", "race_get_efficiency", "race_get_max_stage_depth", "race_get_zone_tree",
    "race_get_phases", "race_get_power_groups", "race_register_function", "race_execute_function",
    "race_execute_function_async", "race_get_status", "race_set_sweep_mode", "race_get_sweep_info", "race_set_power",
    "race_get_power", "race_spmv_plain", "race_spmv_power_layout", "race_get_mpk_layout", "race_set_mpk_schedule",
    "race_mpk_noalloc",
    "race_symmgs_ir", "race_lb_balance", "race_flatten_zone_tree", "race_last_error", "race_register_mpk_block",
    "race_batch_create", "race_batch_destroy", "race_batch_add", "race_batch_prepare", "race_batch_execute",
    "race_batch_graph_launch", "race_batch_get_status", "race_batch_info", "race_batch_last_error",
    "race_mlp_create", "race_mlp_destroy", "race_mlp_num_params", "race_mlp_set_params", "race_mlp_get_params",
    "race_mlp_forward", "race_mlp_loss_grad", "race_mlp_adam_step", "race_mlp_last_error", "race_wave_plan",
    "race_simdify", "race_simdify_schedule", "race_simdify_d1", "race_get_highest_power", "race_get_device_phases",
    "race_zone_tree_host", "race_mpk_stage_partition", "race_mpk_recursion_permute", "race_gather_plan",
    "race_mpk_recursive_partition", "race_set_sub_power", "race_get_sub_power", "race_traverse_host",
    "race_get_power_tree", "race_mpk_issue_order", "race_device_dies",
]


class RaceError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        self.code = code
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")


class race_params(C.Structure):
    _fields_ = [("n_eff", C.c_int), ("eff", C.c_double * 16), ("n_lvl_threads", C.c_int),
                ("lvl_threads", C.c_int * 16), ("cache_violation_cutoff", C.c_int),
                ("max_recursion_stages", C.c_int), ("n_cutoffs", C.c_int), ("cutoffs", C.c_int * 16)]


class race_operands(C.Structure):
    _fields_ = [("n", C.c_int), ("rowPtr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p),
                ("val_type", C.c_int), ("x", C.c_void_p), ("b", C.c_void_p), ("vec_type", C.c_int)]


# callback types of race_zone_tree_host
TRAVERSE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                          C.POINTER(C.c_int))
RANGE_NNZ_FN = C.CFUNCTYPE(C.c_longlong, C.c_void_p, C.c_int, C.c_int)

_lib = None


def lib():
    """The engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"RACE-GB300 engine library missing: {LIB_PATH} (run race_gb300.build.build())")
        L = C.CDLL(str(LIB_PATH))
        vp, ip, i = C.c_void_p, C.POINTER(C.c_int), C.c_int
        sig = {
            "race_params_from_env": [C.POINTER(race_params)],
            "race_create": [C.POINTER(vp), i, i, i, vp, vp, i, vp, vp, i, i, C.POINTER(race_params)],
            "race_destroy": [vp], "race_set_stream": [vp, vp], "race_color": [vp],
            "race_power_prepare": [vp, i, C.c_double, C.c_double, C.c_char_p, i],
            "race_get_perm": [vp, vp, vp], "race_get_num_threads": [vp, ip],
            "race_get_efficiency": [vp, C.POINTER(C.c_double)], "race_get_max_stage_depth": [vp, ip],
            "race_get_zone_tree": [vp, vp, i, ip], "race_get_phases": [vp, i, vp, vp, vp, i, ip, ip],
            "race_get_power_groups": [vp, vp, i, ip],
            "race_register_function": [vp, i, C.POINTER(race_operands), i, ip],
            "race_execute_function": [vp, i, i], "race_execute_function_async": [vp, i, i],
            "race_get_status": [vp], "race_set_power": [vp, i, i], "race_get_power": [vp, i, ip],
            "race_set_sub_power": [vp, i, i], "race_get_sub_power": [vp, i, ip],
            "race_traverse_host": [i, vp, vp, vp, vp, i, i, i, vp, vp, i, ip],
            "race_get_power_tree": [vp, vp, i, ip],
            "race_set_sweep_mode": [vp, i], "race_get_sweep_info": [vp, i, i, ip, ip, ip, ip, ip],
            "race_spmv_plain": [vp, i, vp, vp, vp, vp, vp], "race_spmv_power_layout": [vp, i, i],
            "race_get_mpk_layout": [vp, i, ip, ip, ip, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), ip],
            "race_set_mpk_schedule": [vp, i, i],
            "race_mpk_noalloc": [i, vp, vp, vp, vp, vp, i, i, vp, vp],
            "race_symmgs_ir": [vp, i, i, vp, vp, vp, vp, vp, C.c_double, i, i, ip, C.POINTER(C.c_double)],
            "race_lb_balance": [vp, vp, i, i, C.c_double, i, i, i, i, vp, i, ip],
            "race_flatten_zone_tree": [vp, i, i, i, i, i, i, vp, vp, vp, i, ip, ip],
            "race_register_mpk_block": [vp, C.POINTER(race_operands), i, i, ip],
            "race_batch_create": [C.POINTER(vp)], "race_batch_destroy": [vp], "race_batch_add": [vp, vp, i],
            "race_batch_prepare": [vp, vp], "race_batch_execute": [vp, vp], "race_batch_graph_launch": [vp, vp],
            "race_batch_get_status": [vp, vp], "race_batch_info": [vp, ip, ip, ip],
            "race_mlp_create": [C.POINTER(vp), i, i, i, i], "race_mlp_destroy": [vp],
            "race_mlp_num_params": [vp, C.POINTER(C.c_longlong)], "race_mlp_set_params": [vp, vp, C.c_longlong],
            "race_mlp_get_params": [vp, vp, C.c_longlong], "race_mlp_forward": [vp, vp, i, vp, vp],
            "race_mlp_loss_grad": [vp, vp, vp, i, vp, vp, vp],
            "race_mlp_adam_step": [vp, C.c_float, C.c_float, C.c_float, C.c_float, vp],
            "race_wave_plan": [i, i, vp, vp, vp, vp, vp, i, vp, vp, i, ip, ip],
            "race_simdify": [vp, i, i, i, vp, vp, vp, vp, vp, i, i, ip],
            "race_get_highest_power": [vp, ip],
            "race_get_device_phases": [vp, i, C.POINTER(vp), C.POINTER(vp), ip],
            "race_zone_tree_host": [i, i, i, i, i, C.POINTER(race_params), TRAVERSE_FN, RANGE_NNZ_FN, vp, vp, i, ip,
                                    ip],
            "race_mpk_stage_partition": [vp, vp, i, i, C.c_longlong, i, C.c_double, C.c_double, i, vp, vp, i, ip, ip],
            "race_mpk_recursion_permute": [i, vp, vp, vp, vp, vp, i, vp, i, i],
            "race_mpk_recursive_partition": [i, vp, vp, vp, vp, vp, i, vp, i, i, C.c_longlong, C.c_double, C.c_double,
                                             vp, i, vp, i, ip],
            "race_gather_plan": [i, i, vp, vp, vp, vp, vp, i, vp, vp, vp, i, ip],
            "race_simdify_schedule": [i, i, i, vp, vp, vp, vp, vp, i, i, vp, vp, i, ip],
            "race_simdify_d1": [i, i, i, vp, vp, vp, vp, vp, i, i],
            "race_mpk_issue_order": [vp, vp, vp, i, i, i, i, i, i, i, vp, vp, vp, vp, i, ip],
            "race_device_dies": [ip, vp, i, ip],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.race_last_error.argtypes = [vp]
        L.race_last_error.restype = C.c_char_p
        L.race_batch_last_error.argtypes = [vp]
        L.race_batch_last_error.restype = C.c_char_p
        L.race_mlp_last_error.argtypes = [vp]
        L.race_mlp_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def check(rc: int, handle=None):
    if rc != RACE_SUCCESS:
        msg = ""
        if handle:
            m = lib().race_last_error(handle)
            msg = m.decode() if m else ""
        raise RaceError(rc, msg)
