"""ctypes binding of libhcgpu.so (include/hcgpu.h). Loading fails loudly when the library
is missing: there is no CPU fallback."""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from . import _build

HC_OK = 0
STATUS = {0: "HC_OK", 1: "HC_ERR_INVALID_ARG", 2: "HC_ERR_CUDA", 3: "HC_ERR_NO_SYSTEM",
          4: "HC_ERR_CANCELLED", 5: "HC_ERR_UNSUPPORTED", 6: "HC_ERR_TOO_LARGE", 7: "HC_ERR_TIMEOUT",
          8: "HC_ERR_COMPILE"}
PREC_FP64, PREC_MIXED = 0, 1
STEP_PLAIN, STEP_LEARNED, STEP_EXPLORE = 0, 1, 2


class Options(ct.Structure):
    _fields_ = [
        ("max_steps", ct.c_int32),
        ("extended_precision", ct.c_int32),
        ("max_step_size", ct.c_double),
        ("max_initial_step_size", ct.c_double),
        ("min_step_size", ct.c_double),
        ("min_rel_step_size", ct.c_double),
        ("terminate_cond", ct.c_double),
        ("a", ct.c_double),
        ("beta_a", ct.c_double),
        ("beta_omega_p", ct.c_double),
        ("beta_tau", ct.c_double),
        ("strict_beta_tau", ct.c_double),
        ("min_newton_iters", ct.c_int32),
        ("max_endgame_steps", ct.c_int32),
        ("max_endgame_extended_steps", ct.c_int32),
        ("max_winding_number", ct.c_int32),
        ("zero_is_at_infinity", ct.c_int32),
        ("at_infinity_check", ct.c_int32),
        ("only_nonsingular", ct.c_int32),
        ("refine_steps", ct.c_int32),
        ("endgame_start", ct.c_double),
        ("min_cond", ct.c_double),
        ("min_cond_growth", ct.c_double),
        ("min_coord_growth", ct.c_double),
        ("singular_min_accuracy", ct.c_double),
        ("val_finite_tol", ct.c_double),
        ("val_at_infinity_tol", ct.c_double),
        ("sing_cond", ct.c_double),
        ("sing_accuracy", ct.c_double),
        ("scaling_threshold", ct.c_double),
        ("precision", ct.c_int32),
        ("step_control", ct.c_int32),
        ("warps_per_cta", ct.c_int32),
        ("ctas_per_sm", ct.c_int32),
        ("lockstep", ct.c_int32),
        ("reserved", ct.c_int32),
    ]


RESULT_DTYPE = np.dtype(
    [
        ("return_code", np.int32),
        ("winding_number", np.int32),
        ("t_re", np.float64),
        ("t_im", np.float64),
        ("accuracy", np.float64),
        ("residual", np.float64),
        ("cond", np.float64),
        ("omega", np.float64),
        ("mu", np.float64),
        ("tau", np.float64),
        ("singular", np.int32),
        ("extended_precision", np.int32),
        ("extended_precision_used", np.int32),
        ("_pad", np.int32),
        ("accepted_steps", np.int64),
        ("rejected_steps", np.int64),
        ("steps_eg", np.int64),
        ("path_number", np.int64),
        ("last_t", np.float64),
    ]
)

# exported symbols (kept in sync with include/hcgpu.h; checked by the CPU test suite)
EXPORTS = [
    "hc_default_options", "hc_create", "hc_create_on_device", "hc_destroy", "hc_set_options", "hc_set_homotopy",
    "hc_track", "hc_track_device", "hc_cancel", "hc_set_time_limit", "hc_last_error", "hc_last_stats", "hc_fma_peak",
    "hc_set_step_log", "hc_get_step_log", "hc_track_noalloc", "hc_set_step_model",
    "hc_mlp_num_params", "hc_mlp_forward", "hc_mlp_grad", "hc_mlp_adam",
    "hc_set_slp", "hc_slp_source", "hc_set_slp_parameter_homotopy", "hc_set_slp_parameters", "hc_slp_parameter_source", "hc_set_batch", "hc_set_batch_launch", "hc_autotune_batch", "hc_track_batch_device", "hc_track_batch", "hc_certify", "hc_set_toric", "hc_track_toric", "hc_mixed_cells",
]
STEP_LOG_FIELDS = 36
CERT_DTYPE = np.dtype([("certified", np.int32), ("realness", np.int32), ("radius", np.float64),
                       ("enclosure", np.float64), ("precision", np.int32), ("reserved", np.int32)])

_lib = None


class HCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def load(build_if_missing: bool = True):
    """Load libhcgpu.so (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("HCGPU_LIB") or _build.LIB  # HCGPU_LIB: e.g. a phase-profiling build
    if build_if_missing and path == _build.LIB and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libhcgpu.so not found at {path}; run __graft_entry__.build()")
    L = ct.CDLL(path)
    P = ct.c_void_p
    L.hc_default_options.argtypes = [ct.POINTER(Options)]
    L.hc_create.argtypes = [ct.POINTER(Options), ct.POINTER(P)]
    L.hc_create_on_device.argtypes = [ct.POINTER(Options), ct.c_int, ct.POINTER(P)]
    L.hc_destroy.argtypes = [P]
    L.hc_destroy.restype = None
    L.hc_set_options.argtypes = [P, ct.POINTER(Options)]
    L.hc_set_homotopy.argtypes = [P, ct.c_int, ct.c_int, P, P, P, ct.c_int, P, P, P, ct.c_double, ct.c_double]
    L.hc_set_slp.argtypes = [P, P, P, P, ct.c_double, ct.c_double]
    L.hc_slp_source.argtypes = [P, P, P, P, ct.c_int64, P]
    L.hc_set_slp_parameter_homotopy.argtypes = [P, P, ct.c_int, ct.c_int32, P, P]
    L.hc_set_slp_parameters.argtypes = [P, P, P]
    L.hc_slp_parameter_source.argtypes = [P, ct.c_int, ct.c_int32, P, ct.c_int64, P]
    L.hc_track.argtypes = [P, ct.c_int64, P, ct.c_int, ct.c_double, ct.c_double, ct.c_double, ct.c_double,
                           P, P, P, P]
    L.hc_track_device.argtypes = [P, ct.c_int64, P, ct.c_int, ct.c_double, ct.c_double, ct.c_double,
                                  ct.c_double, P, P, P, P, P]
    L.hc_cancel.argtypes = [P]
    L.hc_set_time_limit.argtypes = [P, ct.c_double]
    L.hc_last_error.argtypes = [P]
    L.hc_last_error.restype = ct.c_char_p
    L.hc_last_stats.argtypes = [P, P, ct.c_int]
    L.hc_fma_peak.argtypes = [P, P]
    L.hc_set_step_log.argtypes = [P, ct.c_int64, ct.c_int64, ct.c_int64]
    L.hc_get_step_log.argtypes = [P, P, ct.c_int64, P]
    L.hc_set_step_model.argtypes = [P, P, P, P, ct.c_double, ct.c_double]
    L.hc_set_batch.argtypes = [P, ct.c_int, P, P, P, P]
    L.hc_set_batch_launch.argtypes = [P, P, P]
    L.hc_autotune_batch.argtypes = [P, P, ct.c_int, P, ct.c_int, ct.c_int, P, P, P]
    L.hc_track_batch_device.argtypes = [P, P, ct.c_int, P, P, P]
    L.hc_track_batch.argtypes = [P, P, ct.c_int, P, P]
    L.hc_certify.argtypes = [P, ct.c_int64, P, ct.c_int, P, P, P]
    L.hc_set_toric.argtypes = [P, ct.c_int, ct.c_int, P, P, P, ct.c_int, P]
    L.hc_track_toric.argtypes = [P, ct.c_int64, P, P, P, P, P, P, P, P]
    L.hc_mixed_cells.argtypes = [ct.c_int, P, P, P, ct.c_int64, P, P, P, P, P]
    L.hc_mlp_num_params.argtypes = []
    L.hc_mlp_forward.argtypes = [P, ct.c_int, P, P, P]
    L.hc_mlp_grad.argtypes = [P, P, P, ct.c_int, P, P, P, P]
    L.hc_mlp_adam.argtypes = [P, P, P, P, ct.c_int, ct.c_float, ct.c_float, P]
    L.hc_track_noalloc.argtypes = [ct.POINTER(Options), ct.c_int, ct.c_int, P, P, P, ct.c_int, P, P, P,
                                   ct.c_double, ct.c_double, ct.c_int64, P, ct.c_int, ct.c_double, ct.c_double,
                                   ct.c_double, ct.c_double, P, P, P]
    _lib = L
    return L


def check(rc, handle=None):
    if rc != HC_OK:
        msg = load().hc_last_error(handle)
        raise HCError(rc, msg.decode() if msg else "")


def default_options(**kw) -> Options:
    o = Options()
    load().hc_default_options(ct.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def ptr(a):
    return None if a is None else a.ctypes.data_as(ct.c_void_p)


def fma_peak():
    """Measured FP64 and FP32 CUDA-core FMA throughput (TFLOP/s) of the current GPU."""
    a = np.zeros(1)
    b = np.zeros(1)
    check(load().hc_fma_peak(ptr(a), ptr(b)))
    return float(a[0]), float(b[0])
