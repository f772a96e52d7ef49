"""ctypes binding of the engine's C ABI (include/bacon_gb300.h).

The shared library must have been built (``python -m bacon_gb300.build_ext``
or ``__graft_entry__.build()``); there is no fallback: loading fails with an
ImportError when the library is absent.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libbacon_gb300.so")

# Status codes (IVPError order, src/ivp.rs:50-76, then extensions).
STATUS_NAMES = {
    0: "Ok",
    1: "MissingParameters",
    2: "UserError",
    3: "ToleranceOOB",
    4: "TimeDeltaOOB",
    5: "TimeEndOOB",
    6: "TimeStartOOB",
    7: "FromPrimitiveFailure",
    8: "MinimumTimeDeltaExceeded",
    9: "MaximumIterationsExceeded",
    10: "SingularMatrix",
    11: "DynamicOnStatic",
    12: "StaticOnDynamic",
    13: "MaxAttemptsExceeded",
    14: "CudaError",
    15: "InvalidArgument",
    16: "Unsupported",
    17: "CapacityExceeded",
}

DP = ctypes.POINTER(ctypes.c_double)
I32P = ctypes.POINTER(ctypes.c_int32)


class Problem(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("dim", ctypes.c_int32),
        ("rhs", ctypes.c_int32),
        ("n_params", ctypes.c_int32),
        ("dyn_dim", ctypes.c_int32),
        ("y0", ctypes.c_void_p),
        ("params", ctypes.c_void_p),
        ("t0", ctypes.c_void_p),
        ("t_end", ctypes.c_void_p),
        ("shared", ctypes.c_void_p),
        ("t0_scalar", ctypes.c_double),
        ("t_end_scalar", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
    ]


class RkOptions(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32),
        ("layout", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("memory", ctypes.c_int32),
        ("max_attempts", ctypes.c_int64),
        ("block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("schedule", ctypes.c_int32),
        ("systems_per_warp", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class RkResult(ctypes.Structure):
    _fields_ = [
        ("y_final", ctypes.c_void_p),
        ("t_final", ctypes.c_void_p),
        ("accepted", ctypes.c_void_p),
        ("rejected", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
        ("traj_t", ctypes.c_void_p),
        ("traj_y", ctypes.c_void_p),
        ("traj_cap", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class BdfOptions(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("memory", ctypes.c_int32),
        ("max_iter", ctypes.c_int32),
        ("max_steps", ctypes.c_int64),
        ("block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
    ]


class AdamsOptions(ctypes.Structure):
    _fields_ = [
        ("order", ctypes.c_int32),
        ("memory", ctypes.c_int32),
        ("max_attempts", ctypes.c_int64),
        ("block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("systems_per_warp", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class RaggedProblem(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("rhs", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("y_offsets", ctypes.c_void_p),
        ("p_offsets", ctypes.c_void_p),
        ("y0", ctypes.c_void_p),
        ("params", ctypes.c_void_p),
        ("t0", ctypes.c_void_p),
        ("t_end", ctypes.c_void_p),
        ("t0_scalar", ctypes.c_double),
        ("t_end_scalar", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
    ]


class RaggedResult(ctypes.Structure):
    _fields_ = [
        ("y_final", ctypes.c_void_p),
        ("t_final", ctypes.c_void_p),
        ("accepted", ctypes.c_void_p),
        ("rejected", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
    ]


class TuneResult(ctypes.Structure):
    _fields_ = [
        ("variant", ctypes.c_int32),
        ("max_registers", ctypes.c_int32),
        ("systems_per_warp", ctypes.c_int32),
        ("block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("candidates", ctypes.c_int32),
        ("best_ms", ctypes.c_double),
        ("default_ms", ctypes.c_double),
    ]


class DenseOutput(ctypes.Structure):
    _fields_ = [
        ("capacity", ctypes.c_int64),
        ("t", ctypes.c_void_p),
        ("y", ctypes.c_void_p),
        ("offsets", ctypes.c_void_p),
        ("total", ctypes.c_int64),
    ]


class RaggedDenseOutput(ctypes.Structure):
    _fields_ = [
        ("capacity", ctypes.c_int64),
        ("value_capacity", ctypes.c_int64),
        ("t", ctypes.c_void_p),
        ("y", ctypes.c_void_p),
        ("offsets", ctypes.c_void_p),
        ("value_offsets", ctypes.c_void_p),
        ("total", ctypes.c_int64),
        ("total_values", ctypes.c_int64),
    ]


class Adjoint(ctypes.Structure):
    _fields_ = [
        ("target", ctypes.c_void_p),
        ("loss", ctypes.c_void_p),
        ("dl_dy0", ctypes.c_void_p),
        ("dl_dp", ctypes.c_void_p),
        ("checkpoint_every", ctypes.c_int32),
        ("max_steps", ctypes.c_int32),
    ]


# Every symbol include/bacon_gb300.h declares, with its ctypes signature.
_VP = ctypes.c_void_p
SIGNATURES = {
    "bacon_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_VP)]),
    "bacon_ctx_destroy": (ctypes.c_int, [_VP]),
    "bacon_last_error": (ctypes.c_char_p, []),
    "bacon_ctx_kernel_launches": (ctypes.c_int64, [_VP]),
    "bacon_ctx_stream": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "bacon_ctx_last_kernel_ms": (ctypes.c_int, [_VP, DP]),
    "bacon_ctx_set_fault_injection": (ctypes.c_int, [_VP, ctypes.c_int]),
    "bacon_rk_solve": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                      ctypes.POINTER(RkResult)]),
    "bacon_rk_solve_user": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                           ctypes.POINTER(RkResult), ctypes.c_void_p, ctypes.c_void_p]),
    "bacon_rk_solve_plain": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                            ctypes.POINTER(RkResult)]),
    "bacon_rk_validate": (ctypes.c_int, [ctypes.POINTER(Problem)]),
    "bacon_bdf_solve": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(BdfOptions),
                                       ctypes.POINTER(RkResult)]),
    "bacon_adams_solve": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(AdamsOptions),
                                         ctypes.POINTER(RkResult)]),
    "bacon_euler_solve": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.c_double,
                                         ctypes.POINTER(AdamsOptions), ctypes.POINTER(RkResult)]),
    "bacon_ragged_validate": (ctypes.c_int, [ctypes.POINTER(RaggedProblem)]),
    "bacon_bdf_solve_mixed": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RaggedProblem),
                                             ctypes.POINTER(BdfOptions), ctypes.POINTER(RkResult),
                                             ctypes.POINTER(RaggedResult)]),
    "bacon_rk_autotune_ex": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                            ctypes.POINTER(RkResult), ctypes.POINTER(TuneResult)]),
    "bacon_rk_set_tuned": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                          ctypes.POINTER(TuneResult)]),
    "bacon_rk_autotune": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                         ctypes.POINTER(RkResult), I32P, I32P]),
    "bacon_rk_solve_adjoint": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                              ctypes.POINTER(RkResult), ctypes.POINTER(Adjoint)]),
    "bacon_ctx_last_reverse_ms": (ctypes.c_int, [_VP, DP]),
    "bacon_rk_solve_dense": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                            ctypes.POINTER(RkResult), ctypes.POINTER(DenseOutput)]),
    "bacon_bdf_solve_dense": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(BdfOptions),
                                             ctypes.POINTER(RkResult), ctypes.POINTER(DenseOutput)]),
    "bacon_euler_solve_dense": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.c_double,
                                               ctypes.POINTER(AdamsOptions), ctypes.POINTER(RkResult),
                                               ctypes.POINTER(DenseOutput)]),
    "bacon_adams_solve_dense": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(AdamsOptions),
                                               ctypes.POINTER(RkResult), ctypes.POINTER(DenseOutput)]),
    "bacon_bdf_solve_mixed_dense": (ctypes.c_int, [_VP, ctypes.POINTER(Problem), ctypes.POINTER(RaggedProblem),
                                                   ctypes.POINTER(BdfOptions), ctypes.POINTER(RkResult),
                                                   ctypes.POINTER(RaggedResult), ctypes.POINTER(DenseOutput),
                                                   ctypes.POINTER(RaggedDenseOutput)]),
    "bacon_rk_solve_noalloc": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(RkOptions),
                                              ctypes.POINTER(RkResult), _VP]),
    "bacon_builder_new": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_VP)]),
    "bacon_builder_new_dyn": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_VP)]),
    "bacon_builder_free": (None, [_VP]),
    "bacon_builder_with_tolerance": (ctypes.c_int, [_VP, ctypes.c_double]),
    "bacon_builder_with_maximum_dt": (ctypes.c_int, [_VP, ctypes.c_double]),
    "bacon_builder_with_minimum_dt": (ctypes.c_int, [_VP, ctypes.c_double]),
    "bacon_builder_with_initial_time": (ctypes.c_int, [_VP, ctypes.c_double]),
    "bacon_builder_with_ending_time": (ctypes.c_int, [_VP, ctypes.c_double]),
    "bacon_builder_with_initial_conditions": (ctypes.c_int, [_VP, DP, ctypes.c_int64]),
    "bacon_builder_with_derivative": (ctypes.c_int, [_VP, ctypes.c_int32, DP, ctypes.c_int32]),
    "bacon_builder_with_ending_times": (ctypes.c_int, [_VP, DP, ctypes.c_int64]),
    "bacon_builder_problem": (ctypes.c_int, [_VP, ctypes.POINTER(Problem)]),
    "bacon_measure_fp64_peak": (ctypes.c_int, [_VP, DP]),
}

_lib = None


def load():
    """Load the engine library (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"bacon_gb300 native library not built: {LIB_PATH} is missing "
                "(run `python -m bacon_gb300.build_ext`)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    msg = load().bacon_last_error()
    return msg.decode() if msg else ""
