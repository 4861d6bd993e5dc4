"""ctypes binding of libcumf_sgd.so (the C ABI declared in include/cumf_sgd.h).

Only plain C types cross the boundary.  The library is loaded from the package's own
lib/ directory; a missing library is an error (there is no fallback implementation).
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libcumf_sgd.so")

CUMF_OK = 0
CUMF_ERR_ARG = 1
CUMF_ERR_IO = 2
CUMF_ERR_FORMAT = 3
CUMF_ERR_CUDA = 4
CUMF_ERR_NOMEM = 5
CUMF_ERR_RANGE = 6
CUMF_ERR_TIMEOUT = 7
CUMF_ERR_NODEVICE = 8

FP16, BF16, FP32, BF16_SR, FP16_SR = 0, 1, 2, 3, 4
PRECISIONS = {"fp16": FP16, "bf16": BF16, "fp32": FP32, "bf16sr": BF16_SR, "fp16sr": FP16_SR}


class Node(C.Structure):
    _fields_ = [("u", C.c_int32), ("v", C.c_int32), ("r", C.c_float)]


class Problem(C.Structure):
    _fields_ = [("m", C.c_int32), ("n", C.c_int32), ("nnz", C.c_int64),
                ("R", C.POINTER(Node)), ("pinned", C.c_int32), ("reserved_", C.c_int32)]


class Params(C.Structure):
    _fields_ = [("k", C.c_int32), ("num_workers", C.c_int32),
                ("u_grid", C.c_int32), ("v_grid", C.c_int32),
                ("x_grid", C.c_int32), ("y_grid", C.c_int32),
                ("ux", C.c_int32), ("vy", C.c_int32),
                ("num_iters", C.c_int32), ("gpu", C.c_int32),
                ("lambda_p", C.c_float), ("lambda_q", C.c_float), ("lrate", C.c_float),
                ("alpha", C.c_float), ("beta", C.c_float),
                ("seed", C.c_uint64), ("precision", C.c_int32), ("lanes", C.c_int32),
                ("quiet", C.c_int32), ("epochs_per_launch", C.c_int32),
                ("verbose_epochs", C.c_int32), ("prefetch", C.c_int32), ("l2_hints", C.c_int32),
                ("ring", C.c_int32), ("tail_epochs", C.c_int32), ("deterministic", C.c_int32),
                ("tail_start", C.c_int64), ("hot_rows", C.c_float), ("reserved_", C.c_int32 * 3)]


class Tuning(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("prefetch", C.c_int32), ("l2_hints", C.c_int32),
                ("ring", C.c_int32), ("freeze_q", C.c_int32), ("rows_copied", C.c_int32),
                ("reserved_", C.c_int32 * 2)]


class Checkpoint(C.Structure):
    _fields_ = [("path", C.c_char_p), ("every", C.c_int32), ("resume", C.c_int32), ("stop_after", C.c_int32),
                ("reserved_", C.c_int32 * 3)]


class Model(C.Structure):
    _fields_ = [("fun", C.c_int32), ("m", C.c_int32), ("n", C.c_int32), ("k", C.c_int32),
                ("b", C.c_float), ("pinned", C.c_int32),
                ("P", C.POINTER(C.c_float)), ("Q", C.POINTER(C.c_float))]


class TrainStats(C.Structure):
    _fields_ = [("prep_ms", C.c_double), ("train_ms", C.c_double), ("export_ms", C.c_double),
                ("total_ms", C.c_double), ("updates_per_sec", C.c_double),
                ("samples_per_epoch", C.c_int64), ("mean", C.c_float), ("std_dev", C.c_float),
                ("mode", C.c_int32), ("num_workers", C.c_int32), ("lanes", C.c_int32),
                ("hot_users", C.c_int32), ("hot_items", C.c_int32), ("extra_rows", C.c_int32),
                ("reserved_", C.c_int32 * 2)]


class BatchProblem(C.Structure):
    _fields_ = [("d_R", C.c_void_p), ("nnz", C.c_int64), ("d_P", C.c_void_p), ("m", C.c_int32), ("n", C.c_int32),
                ("d_Q", C.c_void_p), ("k", C.c_int32), ("num_workers", C.c_int32), ("lambda_p", C.c_float),
                ("lambda_q", C.c_float), ("seed", C.c_uint64), ("d_lr", C.c_void_p), ("lr_len", C.c_int32),
                ("reserved_", C.c_int32), ("hot", C.c_void_p)]


class BatchTuning(C.Structure):
    _fields_ = [("batches_target", C.c_int32), ("order", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("lanes", C.c_int32), ("reserved_", C.c_int32 * 4)]


class Args(C.Structure):
    _fields_ = [("param", Params), ("tr_path", C.c_char * 1024), ("va_path", C.c_char * 1024),
                ("model_path", C.c_char * 1024)]


# name -> (restype, argtypes); every function of include/cumf_sgd.h.
_VP = C.c_void_p
_SIGS = {
    "cumf_abi_version": (C.c_int, []),
    "cumf_hot_rows_per_copy": (C.c_int64, [C.c_int64, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_float]),
    "cumf_hot_rows_plan": (C.c_int, [_VP, C.c_int64, C.c_int32, C.c_int32, C.c_int64, C.c_int32,
                                     C.POINTER(_VP), _VP]),
    "cumf_hot_rows_info": (C.c_int, [_VP, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    "cumf_hot_rows_tables": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "cumf_hot_rows_assign": (C.c_int, [_VP, _VP, C.c_int64, _VP]),
    "cumf_hot_rows_spread": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, _VP]),
    "cumf_hot_rows_merge": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, _VP]),
    "cumf_hot_rows_free": (C.c_int, [_VP]),
    "cumf_last_error": (C.c_char_p, []),
    "cumf_default_params": (C.c_int, [C.POINTER(Params)]),
    "cumf_parse_args": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.POINTER(Args)]),
    "cumf_read_problem": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(Problem)]),
    "cumf_write_problem": (C.c_int, [C.c_char_p, C.POINTER(Problem)]),
    "cumf_train_ckpt": (C.c_int, [C.POINTER(Problem), C.POINTER(Problem), C.POINTER(Params), C.POINTER(Checkpoint),
                                  C.POINTER(Model), C.POINTER(TrainStats), C.POINTER(C.c_int32)]),
    "cumf_selftest_wait_timeout": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "cumf_dev_strata_layout": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cumf_dev_strata_epochs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int32, C.c_void_p,
                                         C.c_int32, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_float,
                                         C.c_float, C.c_uint64, C.c_void_p, C.c_void_p]),
    "cumf_probe_copy_bandwidth": (C.c_int, [C.c_int64, C.c_int, C.POINTER(C.c_double), C.c_void_p]),
    "cumf_evaluate": (C.c_int, [C.POINTER(Problem), C.POINTER(Model), C.c_int, C.POINTER(C.c_double)]),
    "cumf_convert_text": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_int64)]),
    "cumf_read_text_problem": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(Problem)]),
    "cumf_parse_text_host": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "cumf_text_data_start": (C.c_int, [C.c_char_p, C.c_int64, C.c_int, C.POINTER(C.c_int64)]),
    "cumf_dev_parse_text": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int64,
                                      C.POINTER(C.c_int64), C.c_void_p]),
    "cumf_alloc_problem": (C.c_int, [C.c_int64, C.c_int, C.POINTER(Problem)]),
    "cumf_free_problem": (C.c_int, [C.POINTER(Problem)]),
    "cumf_save_model": (C.c_int, [C.POINTER(Model), C.c_char_p]),
    "cumf_load_model": (C.c_int, [C.c_char_p, C.POINTER(Model)]),
    "cumf_alloc_model": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(Model)]),
    "cumf_free_model": (C.c_int, [C.POINTER(Model)]),
    "cumf_train": (C.c_int, [C.POINTER(Problem), C.POINTER(Problem), C.POINTER(Params),
                             C.POINTER(Model), C.POINTER(TrainStats)]),
    "cumf_rmse": (C.c_int, [C.POINTER(Problem), C.POINTER(Model), C.POINTER(C.c_double)]),
    "cumf_lr_schedule": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(C.c_float)]),
    "cumf_batches_per_worker": (C.c_int64, [C.c_int64, C.c_int]),
    "cumf_dev_init_factors": (C.c_int, [_VP, C.c_int64, C.c_int, C.c_int, C.c_uint64, C.c_uint32, _VP]),
    "cumf_sgd_update": (C.c_int, [_VP, C.c_int64, _VP, C.c_int32, _VP, C.c_int32, C.c_int, C.c_int,
                                  C.c_int, C.c_int, _VP, C.c_int, C.c_int, C.c_float, C.c_float,
                                  C.c_uint64, _VP, _VP]),
    "cumf_sgd_update_tuned": (C.c_int, [_VP, C.c_int64, _VP, C.c_int32, _VP, C.c_int32, C.c_int, C.c_int,
                                        C.c_int, C.POINTER(Tuning), _VP, C.c_int, C.c_int, C.c_float,
                                        C.c_float, C.c_uint64, _VP, _VP]),
    "cumf_dev_rating_stats": (C.c_int, [_VP, C.c_int64, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), _VP]),
    "cumf_dev_shuffle_scale": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.c_int32, _VP, C.c_int32,
                                         C.c_float, _VP, _VP]),
    "cumf_dev_export_factors": (C.c_int, [_VP, C.c_int, _VP, C.c_int64, C.c_int, C.c_float, _VP, _VP]),
    "cumf_dev_rmse": (C.c_int, [_VP, C.c_int64, _VP, C.c_int32, _VP, C.c_int32, C.c_int, C.c_float,
                                C.POINTER(C.c_double), _VP]),
    "cumf_dev_rmse_noalloc": (C.c_int, [_VP, C.c_int64, _VP, C.c_int32, _VP, C.c_int32, C.c_int, C.c_float,
                                        C.POINTER(C.c_double), _VP]),
    "cumf_tc_gemm": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, _VP, C.c_int, _VP, C.c_int, C.c_int, _VP,
                               _VP, _VP]),
    "cumf_user_features": (C.c_int, [_VP, C.c_int64, _VP, C.c_int32, C.c_int, C.c_int32, _VP, _VP]),
    "cumf_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]),
    "cumf_mlp_destroy": (C.c_int, [_VP]),
    "cumf_mlp_param_count": (C.c_int64, [_VP]),
    "cumf_mlp_get_params": (C.c_int, [_VP, _VP, C.c_int64, C.c_int]),
    "cumf_mlp_set_params": (C.c_int, [_VP, _VP, C.c_int64]),
    "cumf_mlp_forward": (C.c_int, [_VP, _VP, C.c_int64, _VP, _VP]),
    "cumf_mlp_loss_grad": (C.c_int, [_VP, _VP, _VP, C.c_int64, C.POINTER(C.c_double), _VP]),
    "cumf_mlp_train": (C.c_int, [_VP, _VP, _VP, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64,
                                 C.POINTER(C.c_double), _VP]),
    "cumf_train_ex": (C.c_int, [C.POINTER(Problem), C.POINTER(Problem), C.POINTER(Params), C.POINTER(Model),
                                C.POINTER(Model), C.POINTER(TrainStats), _VP, _VP]),
    "cumf_release_host_cache": (C.c_int, []),
    "cumf_batch_create": (C.c_int, [C.POINTER(BatchProblem), C.c_int, C.POINTER(C.c_void_p)]),
    "cumf_batch_destroy": (C.c_int, [_VP]),
    "cumf_batch_set_tuning": (C.c_int, [_VP, C.POINTER(BatchTuning)]),
    "cumf_batch_get_info": (C.c_int, [_VP, C.POINTER(BatchTuning), C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "cumf_batch_run": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, _VP]),
    "cumf_batch_status": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "cumf_batch_autotune": (C.c_int, [_VP, _VP, C.POINTER(BatchTuning), C.POINTER(C.c_double)]),
    "cumf_device_info": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cumf_default_workers": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int]),
    "cumf_auto_workers": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int]),
    "cumf_random_map": (C.c_int, [C.c_uint32, C.c_int32, C.POINTER(C.c_int32)]),
    "cumf_grid_problem": (C.c_int, [C.POINTER(Node), C.c_int64, C.c_int32, C.c_int32, C.c_int, C.c_int,
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
}

_lib = None


class CumfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cumf error {code}: {msg}")
        self.code = code


def load() -> C.CDLL:
    """Loads the library (build it first with cumf_sgd_gb300.build.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run cumf_sgd_gb300.build.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(rc: int) -> None:
    if rc != CUMF_OK:
        raise CumfError(rc, load().cumf_last_error().decode())


def exported_symbols() -> list[str]:
    return list(_SIGS)
