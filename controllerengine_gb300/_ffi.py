"""ctypes view of include/controller_engine.h.

The library is loaded from the package's in-tree build directory.  There is no
fallback: if libControllerEngine.so is missing or does not load, importing the
engine API raises, so nothing can silently run a CPU path instead.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libControllerEngine.so"

MAX_STATESPACE_DIM = 8
MAX_DISCRETE_DIM = 8
MAX_NONLIN_DIM = 4
MAX_TOTAL_DIM = 16
PRECISION_MIXED = 0
PRECISION_FP64 = 1
PRECISION_COMPENSATED = 2
PRECISION_COMPENSATED_TRAJ64 = 3
PRECISION_COMPENSATED_DF = 4
EIG_ARITH_SEPARATE = 0
EIG_ARITH_FUSED = 1

EXPORTED_SYMBOLS = (
    "ce_last_error", "ce_version", "ce_parse_config", "ce_decode_instructions",
    "ce_session_create", "ce_session_destroy", "ce_session_set_precision", "ce_session_get_config",
    "ce_session_set_eig_arith", "ce_session_get_eig_arith", "ce_evaluate_diagnostics64",
    "ce_evaluate", "ce_evaluate_diagnostics", "ce_evaluate_device", "ce_session_kernel_launches",
    "ce_session_set_profiling", "ce_session_stage_times", "ce_measure_fma_rate", "ce_modal_fit_noalloc",
    "ce_session_set_sim_kernel", "ce_session_sim_kernel", "ce_session_sim_log", "ce_sim_specialised_source",
    "ce_server_create", "ce_server_destroy", "ce_server_submit", "ce_server_wait", "ce_server_get_stats",
    "ce_server_reset_stats", "ce_evaluate_plants", "ce_evaluate_plants_device", "ce_server_create_models",
    "ce_server_submit_model", "ce_server_submit_plants", "ce_session_set_tuning", "ce_session_get_tuning", "ce_session_autotune",
    "ce_ragged_create", "ce_ragged_evaluate", "ce_ragged_destroy", "ce_ragged_kernel_launches",
    "ce_ragged_set_profiling", "ce_ragged_stage_times", "ce_ragged_prepare", "ce_ragged_evaluate_device",
    "ce_ragged_set_tuning", "ce_ragged_get_tuning", "ce_ragged_autotune",
    "RunControllerEngine",
)
PENDING = 2
SIM_TABLE, SIM_SPECIALISED = 0, 1
NUM_STAGES = 6
STAGE_NAMES = ("lina_eig", "sim", "fit", "modal", "nominal", "sweep")


class ce_config(C.Structure):
    _fields_ = [
        ("statespace_dim", C.c_int32), ("discrete_dim", C.c_int32), ("nonlin_dim", C.c_int32),
        ("n_params", C.c_int32), ("input_size", C.c_int32),
        ("dc_instructions", C.c_int32), ("u_instructions", C.c_int32),
        ("nl_instructions", C.c_int32 * MAX_NONLIN_DIM),
        ("n_cores", C.c_int32), ("n_rounds", C.c_int32), ("serial", C.c_int32),
        ("time", C.c_int32), ("duration", C.c_float), ("ref_step_time", C.c_double), ("ref_amplitude", C.c_float),
        ("fit_start", C.c_float), ("fit_end", C.c_float), ("steady_start", C.c_float),
        ("bandwidth", C.c_float), ("damping", C.c_float), ("overshoot", C.c_float),
        ("steady_state_error", C.c_float), ("crossover_coeff", C.c_float), ("target_gm", C.c_float),
        ("target_pm", C.c_float), ("target_b", C.c_float),
        ("eig_fail_err", C.c_float), ("unstable_err", C.c_float),
        ("freq", C.c_int32), ("freq_min", C.c_float), ("dump_diagnostics", C.c_int32),
        ("freq_max_key", C.c_float),
        ("n_threads", C.c_int32), ("freq_max", C.c_float),
        ("total_dim", C.c_int32), ("dc_dim", C.c_int32), ("u_dim", C.c_int32), ("nl_dim", C.c_int32),
        ("nl_instructions_total", C.c_int32),
        ("cuda_mx_width", C.c_int32), ("info_scoring", C.c_int32), ("info_freqresp", C.c_int32),
        ("info_allmargin", C.c_int32), ("info_modal", C.c_int32), ("info_mx_width", C.c_int32),
        ("eigen_mx_width", C.c_int32), ("lina_mx_width", C.c_int32), ("ata_mx_width", C.c_int32),
        ("atb_mx_width", C.c_int32),
        ("ts", C.c_float), ("fit_t0", C.c_float), ("fit_t1", C.c_float), ("damping2", C.c_float),
        ("damping4", C.c_float), ("crossover", C.c_float),
        ("fit_start_id", C.c_int32), ("steady_start_id", C.c_int32), ("fit_steps", C.c_int32),
        ("ref_step_id", C.c_int32), ("observer", C.c_int32),
    ]


class ce_instruction(C.Structure):
    _fields_ = [("op", C.c_int32), ("col", C.c_int32), ("akind", C.c_int32), ("bkind", C.c_int32),
                ("aval", C.c_float), ("bval", C.c_float)]


_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)


class ce_plant(C.Structure):
    _fields_ = [(n, _FP) for n in ("statespace_a", "statespace_a_i", "statespace_b", "statespace_c", "statespace_d",
                                   "discrete_a", "discrete_a_i", "discrete_bu", "discrete_bw", "discrete_c",
                                   "base_params")] + [(n, _IP) for n in ("dc_info", "u_info", "nl_info")]


class ce_diagnostics(C.Structure):
    _fields_ = [(n, _FP) for n in ("yplant", "lina", "eigen", "ata", "atb")]


_DP = C.POINTER(C.c_double)


class ce_diagnostics64(C.Structure):
    _fields_ = [(n, _DP) for n in ("ywin", "summ", "lina", "eigen", "ata", "atb")]


class ce_ragged_tuning(C.Structure):
    _fields_ = [("sim_lanes", C.c_int32), ("instance_order", C.c_int32), ("eig_blocks_per_sm", C.c_int32),
                ("sim_width", C.c_int32), ("ms_per_evaluation", C.c_double)]


class ce_tuning(C.Structure):
    _fields_ = [("eig_lanes", C.c_int32), ("eig_blocks_per_sm", C.c_int32), ("chunks", C.c_int32),
                ("ms_per_evaluation", C.c_double)]


class ce_server_options(C.Structure):
    _fields_ = [("max_batch", C.c_int32), ("lanes", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("max_wait_us", C.c_int32), ("precision", C.c_int32), ("max_batch_work", C.c_int64)]


class ce_server_stats(C.Structure):
    _fields_ = [("capacity", C.c_int64), ("lanes", C.c_int32), ("completed", C.c_int64), ("batches", C.c_int64),
                ("batched_candidates", C.c_int64), ("queued", C.c_int64), ("latency_p50_ms", C.c_double),
                ("latency_p99_ms", C.c_double), ("latency_max_ms", C.c_double), ("queue_p50_ms", C.c_double),
                ("queue_p99_ms", C.c_double), ("service_p50_ms", C.c_double), ("service_p99_ms", C.c_double),
                ("batch_p50_ms", C.c_double), ("batch_p99_ms", C.c_double), ("batch_max_ms", C.c_double),
                ("tail_requests", C.c_int64), ("tail_queue_ms", C.c_double), ("tail_service_ms", C.c_double),
                ("tail_busy_lanes", C.c_double)]


_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libControllerEngine.so (build it first with controllerengine_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m controllerengine_gb300.build` "
                           "(the engine has no CPU fallback)")
    lib = C.CDLL(str(p))
    lib.ce_last_error.restype = C.c_char_p
    lib.ce_version.restype = C.c_char_p
    lib.ce_parse_config.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(ce_config)]
    lib.ce_decode_instructions.argtypes = [_IP, C.c_int32, C.c_int32, _FP, C.c_int32, C.POINTER(ce_instruction)]
    lib.ce_session_create.argtypes = [C.POINTER(ce_config), C.POINTER(ce_plant), C.c_int32, C.POINTER(C.c_void_p)]
    lib.ce_session_destroy.argtypes = [C.c_void_p]
    lib.ce_session_destroy.restype = None
    lib.ce_session_set_precision.argtypes = [C.c_void_p, C.c_int32]
    lib.ce_session_set_eig_arith.argtypes = [C.c_void_p, C.c_int32]
    lib.ce_session_get_eig_arith.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    lib.ce_session_get_config.argtypes = [C.c_void_p, C.POINTER(ce_config)]
    lib.ce_evaluate.argtypes = [C.c_void_p, C.c_int32, C.c_int64, _FP, _FP, _FP]
    lib.ce_evaluate_diagnostics.argtypes = [C.c_void_p, C.c_int32, C.c_int64, _FP, _FP, _FP,
                                            C.POINTER(ce_diagnostics)]
    lib.ce_evaluate_diagnostics64.argtypes = [C.c_void_p, C.c_int32, C.c_int64, _FP, _FP, _FP,
                                              C.POINTER(ce_diagnostics64)]
    lib.ce_evaluate_device.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]
    lib.ce_session_kernel_launches.argtypes = [C.c_void_p]
    lib.ce_session_kernel_launches.restype = C.c_int64
    lib.ce_session_set_sim_kernel.argtypes = [C.c_void_p, C.c_int32]
    lib.ce_session_sim_kernel.argtypes = [C.c_void_p]
    lib.ce_session_sim_kernel.restype = C.c_int32
    lib.ce_session_sim_log.argtypes = [C.c_void_p]
    lib.ce_session_sim_log.restype = C.c_char_p
    lib.ce_sim_specialised_source.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]
    lib.ce_server_create.argtypes = [C.POINTER(ce_config), C.POINTER(ce_plant), C.c_int32,
                                     C.POINTER(ce_server_options), C.POINTER(C.c_void_p)]
    lib.ce_server_create_models.argtypes = [C.POINTER(ce_config), C.POINTER(ce_plant), C.POINTER(C.c_int32), C.c_int32,
                                            C.POINTER(ce_server_options), C.POINTER(C.c_void_p)]
    lib.ce_server_submit_model.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.POINTER(C.c_int64)]
    lib.ce_server_submit_plants.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.POINTER(C.c_int64)]
    lib.ce_session_set_tuning.argtypes = [C.c_void_p, C.POINTER(ce_tuning)]
    lib.ce_session_get_tuning.argtypes = [C.c_void_p, C.POINTER(ce_tuning)]
    lib.ce_session_autotune.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.POINTER(ce_tuning)]
    lib.ce_server_destroy.argtypes = [C.c_void_p]
    lib.ce_server_destroy.restype = None
    lib.ce_ragged_create.argtypes = [C.c_int32, C.POINTER(ce_config), C.POINTER(ce_plant), C.POINTER(C.c_void_p)]
    lib.ce_ragged_evaluate.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ce_ragged_destroy.argtypes = [C.c_void_p]
    lib.ce_ragged_destroy.restype = None
    lib.ce_ragged_kernel_launches.argtypes = [C.c_void_p]
    lib.ce_ragged_kernel_launches.restype = C.c_int64
    lib.ce_ragged_set_profiling.argtypes = [C.c_void_p, C.c_int32]
    lib.ce_ragged_stage_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.ce_ragged_prepare.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    lib.ce_ragged_evaluate_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ce_ragged_set_tuning.argtypes = [C.c_void_p, C.POINTER(ce_ragged_tuning)]
    lib.ce_ragged_get_tuning.argtypes = [C.c_void_p, C.POINTER(ce_ragged_tuning)]
    lib.ce_ragged_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(ce_ragged_tuning)]
    lib.ce_server_submit.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_int64)]
    lib.ce_server_wait.argtypes = [C.c_void_p, C.c_int64, C.c_int32]
    lib.ce_server_get_stats.argtypes = [C.c_void_p, C.POINTER(ce_server_stats)]
    lib.ce_server_reset_stats.argtypes = [C.c_void_p]
    lib.ce_evaluate_plants.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ce_evaluate_plants_device.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p]
    lib.ce_session_set_profiling.argtypes = [C.c_void_p, C.c_int32]
    lib.ce_session_stage_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.ce_measure_fma_rate.argtypes = [C.c_int32, C.POINTER(C.c_double)]
    lib.ce_modal_fit_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int64] + [C.c_void_p] * 6
    lib.RunControllerEngine.restype = C.c_int
    if path is None:
        _lib = lib
    return lib


def last_error(lib: C.CDLL) -> str:
    return lib.ce_last_error().decode(errors="replace")
