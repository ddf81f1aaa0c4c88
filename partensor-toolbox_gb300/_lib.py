"""ctypes binding of libptg.so (the C ABI declared in include/ptg.h).

There is no fallback: if the library cannot be loaded the import of the package's
compute entry points raises."""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libptg.so")
MAX_ORDER = 8

PTG_OK, PTG_ERR_INVALID, PTG_ERR_CUDA, PTG_ERR_OOM, PTG_ERR_UNSUPPORTED, PTG_ERR_TIMEOUT, PTG_ERR_NUMERIC = range(7)
PTG_F32, PTG_BF16, PTG_FP8E4M3 = 0, 1, 2
PTG_OPT_MTTKRP_IMPL = 1
PTG_OPT_NNLS_CLUSTER = 2
PTG_OPT_GTC_ROWS = 3
PTG_OPT_SPIN_LIMIT = 4
PTG_OPT_ALLOC_LIMIT = 5
PTG_OPT_HOST_READ = 6
PTG_OPT_BATCHED_IMPL = 7
MTTKRP_IMPLS = {"auto": 0, "cuda_cores": 1, "tensor_cores": 2}

# every symbol include/ptg.h declares
EXPORTS = [
    "ptg_last_error", "ptg_version", "ptg_ctx_create", "ptg_ctx_destroy", "ptg_ctx_set_stream",
    "ptg_ctx_synchronize", "ptg_ctx_set_option", "ptg_ctx_enable_stats", "ptg_ctx_get_stats", "ptg_ctx_reset_stats",
    "ptg_tensor_create", "ptg_tensor_destroy", "ptg_tensor_norms", "ptg_tensor_storage",
    "ptg_mttkrp", "ptg_cpd_default_options", "ptg_cpd_als", "ptg_cpd",
    "ptg_cpd_dimtree_als", "ptg_cpd_dimtree", "ptg_mttkrp_noalloc", "ptg_cpd_batched",
    "ptg_tensor_create_file", "ptg_cpd_file", "ptg_cpd_dimtree_file",
    "ptg_gtc_default_options", "ptg_gtc", "ptg_gtc_sort_mode",
    "ptg_mlp_create", "ptg_mlp_destroy", "ptg_mlp_num_params", "ptg_mlp_get_params", "ptg_mlp_set_params",
    "ptg_mlp_forward", "ptg_mlp_loss_grad", "ptg_mlp_train",
]


class CpdOptions(ctypes.Structure):
    _fields_ = [("constraints", ctypes.c_int * MAX_ORDER), ("threshold_error", ctypes.c_double),
                ("nesterov_delta_1", ctypes.c_double), ("nesterov_delta_2", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("accel_coeff", ctypes.c_int), ("accel_fail", ctypes.c_int),
                ("acceleration", ctypes.c_int), ("normalization", ctypes.c_int),
                ("refine_sweeps", ctypes.c_int), ("warm_start", ctypes.c_int),
                ("cost_every_sweep", ctypes.c_int), ("warm_model", ctypes.c_void_p),
                ("warm_log_sweeps", ctypes.c_int), ("warm_train_steps", ctypes.c_int),
                ("verify_fp32", ctypes.c_int), ("write_to_file", ctypes.c_int),
                ("final_factors_paths", ctypes.c_char_p * MAX_ORDER)]


class CpdResult(ctypes.Structure):
    _fields_ = [("frob_tns", ctypes.c_double), ("f_value", ctypes.c_double),
                ("rel_costFunction", ctypes.c_double), ("ao_iter", ctypes.c_int),
                ("accel_coeff", ctypes.c_int), ("accel_fail", ctypes.c_int),
                ("refine_sweeps_done", ctypes.c_int), ("nesterov_iters_total", ctypes.c_longlong),
                ("seconds_total", ctypes.c_double)]


class CpdInstance(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("dims", ctypes.c_int64 * MAX_ORDER),
                ("tensor", ctypes.POINTER(ctypes.c_double)), ("rank", ctypes.c_int),
                ("init_factors", ctypes.POINTER(ctypes.POINTER(ctypes.c_double))),
                ("out_factors", ctypes.POINTER(ctypes.POINTER(ctypes.c_double))),
                ("threshold_error", ctypes.c_double)]


class SweepTrace(ctypes.Structure):
    _fields_ = [("f_value", ctypes.c_double), ("rel_costFunction", ctypes.c_double),
                ("f_accel", ctypes.c_double), ("accel_accepted", ctypes.c_int),
                ("nesterov_iters", ctypes.c_int * MAX_ORDER), ("seconds", ctypes.c_float)]


class Stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_longlong), ("mttkrp_launches", ctypes.c_longlong),
                ("mttkrp_ms", ctypes.c_double), ("mttkrp_bytes", ctypes.c_double),
                ("mttkrp_flops", ctypes.c_double), ("tc_launches", ctypes.c_longlong),
                ("tc_ms", ctypes.c_double), ("tc_bytes", ctypes.c_double),
                ("batch_pass_launches", ctypes.c_longlong), ("batch_pass_ms", ctypes.c_double),
                ("batch_pass_bytes", ctypes.c_double)]


class GtcOptions(ctypes.Structure):
    _fields_ = [("constraints", ctypes.c_int * MAX_ORDER), ("threshold_error", ctypes.c_double),
                ("max_nesterov_iter", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("c_stochastic_perc", ctypes.c_double), ("lambdas", ctypes.c_double * MAX_ORDER),
                ("stochastic", ctypes.c_int), ("seed", ctypes.c_ulonglong)]


class GtcResult(ctypes.Structure):
    _fields_ = [("frob_tns", ctypes.c_double), ("f_value", ctypes.c_double),
                ("rel_costFunction", ctypes.c_double), ("ao_iter", ctypes.c_int), ("epochs", ctypes.c_int),
                ("seconds_setup", ctypes.c_double), ("seconds_total", ctypes.c_double)]


class PtgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ptg error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libptg.so (raises OSError when it is missing: build it with build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(path)
    vp, i64p, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)
    dpp = ctypes.POINTER(dp)
    lib.ptg_last_error.restype = ctypes.c_char_p
    lib.ptg_version.restype = ctypes.c_char_p
    lib.ptg_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    lib.ptg_ctx_destroy.argtypes = [vp]
    lib.ptg_ctx_set_stream.argtypes = [vp, vp]
    lib.ptg_ctx_synchronize.argtypes = [vp]
    lib.ptg_ctx_set_option.argtypes = [vp, ctypes.c_int, ctypes.c_longlong]
    lib.ptg_ctx_enable_stats.argtypes = [vp, ctypes.c_int]
    lib.ptg_ctx_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.ptg_ctx_reset_stats.argtypes = [vp]
    lib.ptg_tensor_create.argtypes = [vp, ctypes.c_int, i64p, ctypes.c_int, dp, ctypes.c_int, ctypes.POINTER(vp)]
    lib.ptg_tensor_destroy.argtypes = [vp]
    lib.ptg_tensor_norms.argtypes = [vp, dp, dp]
    lib.ptg_tensor_storage.argtypes = [vp, ctypes.POINTER(vp), i64p, ctypes.POINTER(vp)]
    lib.ptg_mttkrp.argtypes = [vp, vp, ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, vp]
    lib.ptg_cpd_default_options.argtypes = [ctypes.c_int, ctypes.POINTER(CpdOptions)]
    lib.ptg_cpd_default_options.restype = None
    lib.ptg_cpd_als.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.POINTER(CpdOptions), dpp, dpp,
                                ctypes.POINTER(CpdResult), ctypes.POINTER(SweepTrace)]
    lib.ptg_cpd.argtypes = [vp, ctypes.c_int, i64p, dp, ctypes.c_int, ctypes.c_int,
                            ctypes.POINTER(CpdOptions), dpp, dpp, ctypes.POINTER(CpdResult),
                            ctypes.POINTER(SweepTrace)]
    lib.ptg_mttkrp_noalloc.argtypes = [vp, ctypes.c_int, i64p, ctypes.c_int64, ctypes.POINTER(vp),
                                       ctypes.c_int, ctypes.c_int, vp, vp]
    lib.ptg_gtc_default_options.argtypes = [ctypes.c_int, ctypes.POINTER(GtcOptions)]
    lib.ptg_gtc_default_options.restype = None
    lib.ptg_gtc.argtypes = [vp, ctypes.c_int, i64p, ctypes.c_int64, vp, vp, ctypes.c_int, ctypes.c_int,
                            ctypes.POINTER(GtcOptions), dpp, dpp, ctypes.POINTER(GtcResult),
                            ctypes.POINTER(SweepTrace)]
    lib.ptg_gtc_sort_mode.argtypes = [vp, ctypes.c_int, i64p, ctypes.c_int64, vp, ctypes.c_int, vp]
    lib.ptg_mlp_create.argtypes = [vp, ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(vp)]
    lib.ptg_mlp_destroy.argtypes = [vp]
    lib.ptg_mlp_num_params.argtypes = [vp]
    lib.ptg_mlp_num_params.restype = ctypes.c_longlong
    lib.ptg_mlp_get_params.argtypes = [vp, vp, vp]
    lib.ptg_mlp_set_params.argtypes = [vp, vp, vp]
    lib.ptg_mlp_forward.argtypes = [vp, vp, vp, ctypes.c_longlong, vp]
    lib.ptg_mlp_loss_grad.argtypes = [vp, vp, vp, vp, ctypes.c_int, dp, vp]
    lib.ptg_mlp_train.argtypes = [vp, vp, vp, vp, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                  ctypes.c_ulonglong, dp]
    lib.ptg_cpd_dimtree_als.argtypes = lib.ptg_cpd_als.argtypes
    cpp = ctypes.POINTER(ctypes.c_char_p)
    lib.ptg_tensor_create_file.argtypes = [vp, ctypes.c_int, i64p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int64,
                                           ctypes.POINTER(vp)]
    lib.ptg_cpd_file.argtypes = [vp, ctypes.c_int, i64p, ctypes.c_char_p, ctypes.c_int64, cpp, ctypes.c_ulonglong,
                                 ctypes.c_int, ctypes.c_int, ctypes.POINTER(CpdOptions), dpp,
                                 ctypes.POINTER(CpdResult), ctypes.POINTER(SweepTrace)]
    lib.ptg_cpd_dimtree_file.argtypes = lib.ptg_cpd_file.argtypes
    lib.ptg_cpd_batched.argtypes = [vp, ctypes.c_int, ctypes.POINTER(CpdInstance), ctypes.POINTER(CpdOptions),
                                    ctypes.POINTER(CpdResult), dp]
    lib.ptg_cpd_dimtree.argtypes = lib.ptg_cpd.argtypes
    for name in EXPORTS:
        if name not in ("ptg_last_error", "ptg_version", "ptg_cpd_default_options", "ptg_gtc_default_options",
                        "ptg_mlp_num_params"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def check(code: int):
    if code != PTG_OK:
        raise PtgError(code, load().ptg_last_error().decode())
