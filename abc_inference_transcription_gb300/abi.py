"""ctypes mirror of include/abcgpu.h and the loader of libabcgpu.so.

The structures here are byte-for-byte the C structs of the ABI; the oracle's
test wrapper reuses them.  Loading the library never falls back to anything:
if libabcgpu.so is missing the import of the product path fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

MAX_AGES = 8
MAX_CONDS = 16
MAX_STEPS = 8
MAX_PARAMS = 32

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_EVENT_CAP = -4
ERR_NONFINITE = -5
ERR_CAPACITY = -6
ERR_STATE = -7
ERR_IO = -8

STATUS_NAMES = {
    OK: "ABC_OK", ERR_INVALID: "ABC_ERR_INVALID", ERR_CUDA: "ABC_ERR_CUDA",
    ERR_NOMEM: "ABC_ERR_NOMEM", ERR_EVENT_CAP: "ABC_ERR_EVENT_CAP",
    ERR_NONFINITE: "ABC_ERR_NONFINITE", ERR_CAPACITY: "ABC_ERR_CAPACITY",
    ERR_STATE: "ABC_ERR_STATE", ERR_IO: "ABC_ERR_IO",
}

# model index m of wrapper.jl:47-51
MODEL_NAMES = ["const", "const_const", "kon", "alpha", "gamma"]
FP64 = 0
FP32 = 1


class AbcConfig(C.Structure):
    _fields_ = [
        ("cycle", C.c_double),
        ("n_burn_cycles", C.c_int32),
        ("n_steps", C.c_int32),
        ("n_ages", C.c_int32),
        ("n_conds", C.c_int32),
        ("ages", C.c_double * MAX_AGES),
        ("pulse", C.c_double * MAX_CONDS),
        ("chase", C.c_double * MAX_CONDS),
        ("pulse_stat_cond", C.c_int32),
        ("chase_stat_cond", C.c_int32),
        ("splicing", C.c_int32),
        ("scaling_column", C.c_int32),
        ("precision", C.c_int32),
        ("reserved0", C.c_int32),
        ("event_cap", C.c_int64),
    ]


class AbcPrior(C.Structure):
    _fields_ = [
        ("kon", C.c_double * 2), ("koff", C.c_double * 2), ("alpha", C.c_double * 2),
        ("gamma", C.c_double * 2), ("lambda_", C.c_double * 2), ("beta", C.c_double * 2),
        ("scaling", C.c_double * 2), ("vary_mode", C.c_int32), ("reserved0", C.c_int32),
        ("factor", C.c_double * 2),
    ]


def nstats(n_ages: int, n_conds: int) -> int:
    """4A + 3J, scripts/compute_errors.jl:51."""
    return 4 * n_ages + 3 * n_conds


def breakpoint_grid(cfg: AbcConfig) -> float | None:
    """The power-of-two quantum on which every time of cfg lies (the production
    SSA then places breakpoints with integer arithmetic), or None."""
    q = C.c_double(0.0)
    st = load_library().abc_breakpoint_grid(C.byref(cfg), C.byref(q))
    if st < 0:
        raise AbcError(st, "invalid configuration")
    return q.value if st == 1 else None


def num_params(cfg: AbcConfig, model: int) -> int:
    """theta columns: get_vary_map (scripts/model.jl:30-43) + lambda + extensions."""
    if model not in (1, 2, 3, 4, 5):
        raise ValueError(f"model must be 1..5, got {model}")
    return 5 + (cfg.n_steps - 1 if model >= 3 else 0) + int(bool(cfg.splicing)) + int(bool(cfg.scaling_column))


def ptr(a: np.ndarray | None, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libabcgpu.so")


class AbcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load libabcgpu.so (built by abc_inference_transcription_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            f"{p} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = C.CDLL(p)
    _declare(lib)
    if path is None:
        _lib = lib
    return lib


def _declare(lib: C.CDLL) -> None:
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    i32p = C.POINTER(C.c_int32)
    i64p = C.POINTER(C.c_int64)
    u64p = C.POINTER(C.c_uint64)
    i64 = C.c_int64
    u64 = C.c_uint64
    sig = {
        "abc_create": (C.c_int, [C.POINTER(vp), C.POINTER(AbcConfig)]),
        "abc_destroy": (C.c_int, [vp]),
        "abc_last_error": (C.c_char_p, [vp]),
        "abc_num_params": (C.c_int, [vp, C.c_int]),
        "abc_num_stats": (C.c_int, [vp]),
        "abc_stream": (vp, [vp]),
        "abc_set_cells": (C.c_int, [vp, i64, i32p, i32p, dp, dp]),
        "abc_sample_prior": (C.c_int, [vp, C.c_int, i64, u64, i64, C.POINTER(AbcPrior), dp]),
        "abc_sample_prior_device": (C.c_int, [vp, C.c_int, i64, u64, i64, C.POINTER(AbcPrior), vp]),
        "abc_simulate": (C.c_int, [vp, C.c_int, dp, i64, u64, i64, dp]),
        "abc_simulate_device": (C.c_int, [vp, C.c_int, vp, i64, u64, i64, vp]),
        "abc_synchronize": (C.c_int, [vp]),
        "abc_simulate_batch": (C.c_int, [vp, i32p, dp, i64, i64, u64, i64, dp]),
        "abc_simulate_batch_device": (C.c_int, [vp, vp, vp, i64, i64, u64, i64, vp]),
        "abc_simulate_noalloc": (C.c_int, [C.POINTER(AbcConfig), C.c_int, i64, i32p, i32p, dp, dp, vp, i64, u64,
                                           i64, vp, vp]),
        "abc_simulate_cells": (C.c_int, [vp, C.c_int, dp, i64, u64, i64, i32p, i32p, i64p, u64p, dp]),
        "abc_last_counters": (C.c_int, [vp, i64p, i64p]),
        "abc_profile": (C.c_int, [vp, C.c_int]),
        "abc_autotune": (C.c_int, [vp, C.c_int, dp, i64, u64, dp, C.POINTER(C.c_int)]),
        "abc_set_variant": (C.c_int, [vp, C.c_int]),
        "abc_autotune_batch": (C.c_int, [vp, i32p, dp, i64, i64, u64, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "abc_set_work_chunk": (C.c_int, [vp, C.c_int]),
        "abc_profile_read": (C.c_int, [vp, dp]),
        "abc_errors": (C.c_int, [vp, dp, dp, i64, C.c_int, C.c_int, i32p, dp, i64, dp]),
        "abc_errors_select": (C.c_int, [vp, dp, dp, i64, C.c_int, C.c_int, i32p, dp, i64, C.c_int,
                                        C.c_double, i64p]),
        "abc_errors_select_thr": (C.c_int, [vp, dp, dp, i64, C.c_int, C.c_int, i32p, dp, i64, dp, i64p]),
        "abc_errors_select_device": (C.c_int, [vp, dp, dp, i64, C.c_int, C.c_int, i32p, vp, i64, C.c_int,
                                               C.c_double, dp, i64p]),
        "abc_accept_fetch": (C.c_int, [vp, i64p, i64p, dp]),
        "abc_select_counters": (C.c_int, [vp, i64p, i64p]),
        "abc_set_select_errors": (C.c_int, [vp, C.c_int]),
        "abc_accept_errors": (C.c_int, [vp, dp]),
        "abc_breakpoint_grid": (C.c_int, [C.POINTER(AbcConfig), dp]),
        "abc_write_particles": (C.c_int, [C.c_char_p, C.c_int, C.c_int64, i64p, i64p]),
        "abc_write_matrix": (C.c_int, [C.c_char_p, C.c_int, C.c_int64, C.c_int64, dp, C.c_int64]),
        "abc_format_double": (C.c_int, [C.c_double, C.c_char_p, C.c_int]),
        "abc_read_particles": (C.c_int, [C.c_char_p, i64p, i64p, i64p, i64p]),
        "abc_select_profile_read": (C.c_int, [vp, dp, C.POINTER(C.c_int)]),
        "abc_set_distance_mode": (C.c_int, [vp, C.c_int]),
        "abc_set_graph": (C.c_int, [vp, C.c_int]),
        "abc_graph_counters": (C.c_int, [vp, i64p, i64p]),
        "abc_moment_simulate": (C.c_int, [vp, C.c_int, dp, C.c_int64, dp, C.c_double, dp, C.c_int, dp, dp, dp,
                                          C.POINTER(C.c_int32)]),
        "abc_data_stats": (C.c_int, [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int64, C.c_int,
                                     C.c_uint64, dp, dp]),
        "abc_model_probs": (C.c_int, [vp, i64p, C.c_int64, C.c_int, C.c_int, C.c_double, C.c_uint64, dp, dp, dp]),
        "abc_posterior_summary": (C.c_int, [vp, dp, C.c_int64, C.c_int, C.c_int, C.c_double, dp, dp, dp, dp,
                                            i64p]),
        "abc_get_distance_mode": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "abc_errors_candidate": (C.c_int, [vp, dp, dp, C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_int32), dp,
                                           C.c_int64, C.POINTER(C.c_float), dp, dp, C.POINTER(C.c_int)]),
    }
    sp = vp
    sig.update({
        "abc_surrogate_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int, C.c_int, u64]),
        "abc_surrogate_destroy": (C.c_int, [sp]),
        "abc_surrogate_last_error": (C.c_char_p, [sp]),
        "abc_surrogate_num_params": (C.c_int, [sp]),
        "abc_surrogate_set_screen_mode": (C.c_int, [sp, C.c_int]),
        "abc_surrogate_train": (C.c_int, [sp, dp, dp, i64, C.c_int, C.c_int, C.c_double, dp]),
        "abc_surrogate_gradients": (C.c_int, [sp, dp, dp, i64, dp, C.POINTER(C.c_float)]),
        "abc_surrogate_get_params": (C.c_int, [sp, C.POINTER(C.c_float)]),
        "abc_surrogate_set_params": (C.c_int, [sp, C.POINTER(C.c_float)]),
        "abc_surrogate_get_norm": (C.c_int, [sp, dp, dp, dp, dp]),
        "abc_surrogate_set_norm": (C.c_int, [sp, dp, dp, dp, dp]),
        "abc_surrogate_predict": (C.c_int, [sp, dp, i64, dp, dp, dp]),
        "abc_surrogate_predict_device": (C.c_int, [sp, vp, C.c_int, i64, vp, vp, vp]),
        "abc_surrogate_compact_device": (C.c_int, [sp, vp, vp, C.c_int, i64, vp, vp, i64p]),
        "abc_surrogate_screen_device": (C.c_int, [sp, vp, C.c_int, i64, dp, dp, i64, dp, C.c_double, C.c_double,
                                                  C.c_double, vp, i64p, dp]),
    })
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


# Every symbol include/abcgpu.h declares (checked by the CPU test suite).
ABI_SYMBOLS = [
    "abc_create", "abc_destroy", "abc_last_error", "abc_num_params", "abc_num_stats",
    "abc_stream", "abc_set_cells", "abc_sample_prior", "abc_sample_prior_device", "abc_simulate", "abc_simulate_device",
    "abc_synchronize", "abc_simulate_batch", "abc_simulate_batch_device", "abc_simulate_noalloc", "abc_simulate_cells", "abc_last_counters",
    "abc_profile", "abc_profile_read", "abc_autotune", "abc_autotune_batch", "abc_set_variant",
    "abc_set_work_chunk", "abc_errors",
    "abc_errors_select", "abc_errors_select_thr", "abc_errors_select_device", "abc_accept_fetch",
    "abc_select_counters", "abc_select_profile_read", "abc_set_select_errors", "abc_accept_errors", "abc_breakpoint_grid", "abc_write_particles", "abc_write_matrix",
    "abc_format_double", "abc_read_particles", "abc_set_distance_mode", "abc_get_distance_mode",
    "abc_errors_candidate", "abc_model_probs", "abc_posterior_summary",
    "abc_moment_simulate", "abc_data_stats", "abc_set_graph", "abc_graph_counters",
    "abc_surrogate_create", "abc_surrogate_destroy", "abc_surrogate_last_error", "abc_surrogate_num_params",
    "abc_surrogate_train", "abc_surrogate_gradients", "abc_surrogate_get_params", "abc_surrogate_set_params",
    "abc_surrogate_get_norm", "abc_surrogate_set_norm", "abc_surrogate_predict", "abc_surrogate_predict_device",
    "abc_surrogate_screen_device", "abc_surrogate_compact_device", "abc_surrogate_set_screen_mode",
]
