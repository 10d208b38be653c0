"""ctypes binding of the engine's C ABI (include/superdca_gb300.h).

The library is built in-tree by superdca_gb300/build.py.  There is no CPU
fallback: loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsuperdca_gb300.so")

SDCA_OK = 0
SDCA_E_ARG = -1
SDCA_E_CUDA = -2
SDCA_E_STATE = -3
SDCA_E_NOMEM = -4
SDCA_E_NUMERIC = -5
SDCA_E_UNSUPPORTED = -6

FORM_GATHER = 0
FORM_TC = 1
FORM_DUAL = 2
FLAG_HISTORY_BF16 = 0x1

K_FORWARD, K_BACKWARD, K_LINESEARCH, K_HISTORY, K_DIRECTION, K_ACCEPT, K_SCORE, K_OTHER = range(8)
KERNEL_CLASSES = ["forward", "backward", "linesearch", "history", "direction", "accept", "score",
                  "other"]

# every entry point include/superdca_gb300.h declares
EXPORTS = ["sdca_abi_version", "sdca_config_default", "sdca_create", "sdca_set_alignment",
           "sdca_compute_weights", "sdca_get_lambdas", "sdca_solve", "sdca_solve_ex", "sdca_solve_sel", "sdca_eval",
           "sdca_get_profile", "sdca_last_error", "sdca_destroy", "sdca_eval_noalloc",
           "sdca_set_warm_start", "sdca_ws_features", "sdca_mlp_blob_size", "sdca_mlp_grad",
           "sdca_mlp_predict", "sdca_mlp_train", "sdca_mlp_last_error", "sdca_set_targets", "sdca_autotune",
           "sdca_ws_dual_data"]


class Config(C.Structure):
    _fields_ = [("n_seqs", C.c_int64), ("n_loci", C.c_int64), ("q", C.c_int32),
                ("gap_state", C.c_int32), ("lambda_h", C.c_double), ("lambda_J", C.c_double),
                ("gradient_threshold", C.c_double), ("max_iterations", C.c_int32),
                ("history", C.c_int32), ("batch", C.c_int32), ("form", C.c_int32),
                ("flags", C.c_int32), ("device", C.c_int32), ("stream", C.c_void_p),
                ("lanes", C.c_int32), ("reserved0", C.c_int32)]


class LocusStat(C.Structure):
    _fields_ = [("f", C.c_double), ("gnorm", C.c_double), ("iterations", C.c_int32),
                ("nfeval", C.c_int32), ("contractions", C.c_int32), ("status", C.c_int32),
                ("restarts", C.c_int32), ("skipped_pairs", C.c_int32), ("weak_searches", C.c_int32),
                ("max_trials", C.c_int32)]


class TuneEntry(C.Structure):
    _fields_ = [("batch", C.c_int32), ("lanes", C.c_int32), ("n_loci", C.c_int32), ("status", C.c_int32),
                ("device_ms", C.c_double), ("iterations_per_s", C.c_double)]


TUNE_MAX_ENTRIES = 16


class Profile(C.Structure):
    _fields_ = [("solve_ms", C.c_double), ("kernel_ms", C.c_double * 8),
                ("kernel_launches", C.c_int64 * 8), ("kernel_units", C.c_int64 * 8),
                ("gpu_launches", C.c_int64), ("iterations", C.c_int64),
                ("contractions", C.c_int64), ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64)]


_lib = None


def load(path: str = LIB_PATH):
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"engine library {path} is missing: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    vp, i64, dp = C.c_void_p, C.c_int64, C.c_double
    L.sdca_abi_version.restype = C.c_int
    L.sdca_config_default.argtypes = [C.POINTER(Config)]
    L.sdca_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
    L.sdca_set_alignment.argtypes = [vp, vp, vp]
    L.sdca_compute_weights.argtypes = [vp, vp, vp, dp, vp]
    L.sdca_get_lambdas.argtypes = [vp, C.POINTER(dp), C.POINTER(dp), C.POINTER(dp)]
    L.sdca_solve.argtypes = [vp, vp, C.c_size_t, vp, vp]
    L.sdca_solve_ex.argtypes = [vp, vp, C.c_size_t, vp, vp, vp, vp]
    L.sdca_solve_sel.argtypes = [vp, vp, C.c_size_t, vp, vp, vp, vp, vp]
    L.sdca_eval.argtypes = [vp, C.c_uint32, vp, C.POINTER(dp), vp]
    L.sdca_get_profile.argtypes = [vp, C.POINTER(Profile)]
    L.sdca_last_error.restype = C.c_char_p
    L.sdca_last_error.argtypes = [vp]
    L.sdca_destroy.argtypes = [vp]
    L.sdca_eval_noalloc.argtypes = [vp, i64, i64, vp, dp, dp, C.c_uint32, vp, vp, vp, vp]
    L.sdca_set_warm_start.argtypes = [vp, vp, C.c_size_t]
    L.sdca_set_targets.argtypes = [vp, vp, i64]
    L.sdca_ws_dual_data.argtypes = [vp, vp, C.c_size_t, vp, vp, vp]
    L.sdca_autotune.argtypes = [C.POINTER(Config), vp, vp, vp, C.c_size_t, dp, C.c_char_p, vp, vp,
                                C.POINTER(C.c_size_t), C.POINTER(Config), vp, C.POINTER(C.c_int32)]
    L.sdca_ws_features.argtypes = [vp, C.c_int, C.c_float, vp, C.c_size_t, vp, C.c_size_t, vp]
    L.sdca_mlp_blob_size.argtypes = []
    L.sdca_mlp_grad.argtypes = [vp, vp, vp, i64, C.POINTER(dp), vp]
    L.sdca_mlp_predict.argtypes = [vp, vp, i64, vp]
    L.sdca_mlp_train.argtypes = [vp, vp, vp, i64, C.c_int, C.c_int, C.c_float, C.c_uint64, vp]
    L.sdca_mlp_last_error.restype = C.c_char_p
    L.sdca_mlp_last_error.argtypes = []
    L.sdca_internal_lbfgs_coeffs.argtypes = [C.c_int, vp, vp, vp, vp, dp, C.POINTER(dp), vp, vp]
    for name in EXPORTS + ["sdca_internal_lbfgs_coeffs"]:
        if name not in ("sdca_abi_version", "sdca_last_error", "sdca_mlp_last_error"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"superdca_gb300 error {code}: {msg}")
        self.code = code
