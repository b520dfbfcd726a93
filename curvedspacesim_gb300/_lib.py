"""ctypes binding of libcssg.so (the C ABI declared in include/cssg.h).

The library is the only compute path: if it is missing or fails to load this module raises, there is no fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_lib = None

CSSG_OK = 0
STATUS_NAMES = {0: "ok", 1: "border", 2: "nan", 3: "vertex", 4: "iteration cap", 5: "no intersection",
                6: "capacity"}

# every entry point declared in include/cssg.h
EXPORTS = [
    "cssg_last_error", "cssg_version", "cssg_mesh_create", "cssg_mesh_destroy", "cssg_mesh_info", "cssg_ctx_create",
    "cssg_ctx_destroy", "cssg_ctx_synchronize", "cssg_ctx_stream", "cssg_transport_batch", "cssg_distance_batch",
    "cssg_system_create", "cssg_system_destroy", "cssg_system_set_state", "cssg_system_get_state",
    "cssg_system_device_state", "cssg_system_step", "cssg_system_compute_forces", "cssg_system_check",
    "cssg_system_pairs", "cssg_system_chain", "cssg_system_timing", "cssg_system_last_times",
    "cssg_system_reset_thermostat", "cssg_system_kernels_per_step", "cssg_diag_fp64_peak",
    "cssg_system_create_batched", "cssg_mlp_param_count", "cssg_screen_features", "cssg_mlp_infer", "cssg_mlp_grad",
    "cssg_mlp_adam", "cssg_system_set_screen", "cssg_system_screen_counters", "cssg_distance_batch_noalloc",
    "cssg_system_set_tuning", "cssg_system_autotune", "cssg_system_fire", "cssg_system_stress",
    "cssg_mesh_set_boundary", "cssg_diag_reciprocal", "cssg_system_step_host",
    "cssg_system_gradient_descent", "cssg_system_set_screen_audit", "cssg_system_screen_audit_status",
    "cssg_system_set_work_caps", "cssg_system_set_lanes", "cssg_system_lanes", "cssg_diag_flops_per_window",
    "cssg_system_set_lane_split", "cssg_system_lane_split", "cssg_system_source_costs", "cssg_system_set_pass_groups",
    "cssg_system_pass_groups", "cssg_system_kernels_per_audit_step",
]


class cssg_params(ctypes.Structure):
    _fields_ = [
        ("integrator", ctypes.c_int),
        ("force_kind", ctypes.c_int),
        ("k", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("range", ctypes.c_double),
        ("submesh", ctypes.c_int),
        ("max_dist", ctypes.c_double),
        ("cutoff", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("temperature", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("chain_length", ctypes.c_int),
    ]


class cssg_fire_params(ctypes.Structure):
    _fields_ = [
        ("maximum_iterations", ctypes.c_int),
        ("alpha_start", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_inc", ctypes.c_double),
        ("dt_dec", ctypes.c_double),
        ("alpha_dec", ctypes.c_double),
        ("n_min", ctypes.c_int),
        ("force_cutoff", ctypes.c_double),
        ("alpha_min", ctypes.c_double),
    ]


class CssgError(RuntimeError):
    pass


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libcssg.so (building it first when it is absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise CssgError(f"libcssg.so not built ({path})")
        _build.build()
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I = ctypes.c_int
    D = ctypes.c_double
    PP = ctypes.POINTER(ctypes.c_void_p)
    L.cssg_last_error.restype = ctypes.c_char_p
    L.cssg_version.restype = ctypes.c_char_p
    L.cssg_mesh_create.argtypes = [P, I, P, I, I, PP]
    L.cssg_mesh_destroy.argtypes = [P]
    L.cssg_mesh_info.argtypes = [P, P, P, P, P]
    L.cssg_mesh_set_boundary.argtypes = [P, I]
    L.cssg_ctx_create.argtypes = [I, P, PP]
    L.cssg_ctx_destroy.argtypes = [P]
    L.cssg_ctx_synchronize.argtypes = [P]
    L.cssg_ctx_stream.argtypes = [P]
    L.cssg_ctx_stream.restype = P
    L.cssg_transport_batch.argtypes = [P, P, I, P, P, P, P, I, P, P]
    L.cssg_distance_batch.argtypes = [P, P, I, P, P, P, P, P, I, D, P, D, P, P, P, P, P]
    L.cssg_distance_batch_noalloc.argtypes = [P, P, I, P, P, P, P, P, I, D, P, D, P, P, P, P, P]
    L.cssg_system_create.argtypes = [P, P, I, ctypes.POINTER(cssg_params), PP]
    L.cssg_system_create_batched.argtypes = [P, I, P, P, P, PP]
    L.cssg_system_destroy.argtypes = [P]
    L.cssg_system_set_state.argtypes = [P, P, P, P, P]
    L.cssg_system_get_state.argtypes = [P, P, P, P, P]
    L.cssg_system_device_state.argtypes = [P, PP, PP, PP, PP]
    L.cssg_system_step.argtypes = [P, I, I]
    L.cssg_system_step_host.argtypes = [P, I, P, P, P, P, P, P, P, P]
    L.cssg_system_gradient_descent.argtypes = [P, I, D, I]
    L.cssg_system_compute_forces.argtypes = [P]
    L.cssg_system_set_tuning.argtypes = [P, D, I, I, I, I, I, I]
    L.cssg_system_autotune.argtypes = [P, I, P]
    L.cssg_system_fire.argtypes = [P, ctypes.POINTER(cssg_fire_params), I, P]
    L.cssg_system_stress.argtypes = [P, P]
    L.cssg_system_check.argtypes = [P, P, P]
    L.cssg_system_pairs.argtypes = [P, I, P, P, P, P, P]
    L.cssg_system_chain.argtypes = [P, P, I]
    L.cssg_system_timing.argtypes = [P, I]
    L.cssg_system_last_times.argtypes = [P, P, I]
    L.cssg_system_reset_thermostat.argtypes = [P]
    L.cssg_system_kernels_per_step.argtypes = [P, P]
    L.cssg_diag_fp64_peak.argtypes = [P, P]
    L.cssg_diag_reciprocal.argtypes = [P, I, P, P]
    L.cssg_diag_flops_per_window.argtypes = []
    L.cssg_mlp_param_count.argtypes = []
    L.cssg_system_set_screen.argtypes = [P, P, D, I]
    L.cssg_system_screen_counters.argtypes = [P, P]
    L.cssg_system_set_screen_audit.argtypes = [P, I]
    L.cssg_system_set_work_caps.argtypes = [P, I, I, I]
    L.cssg_system_set_lanes.argtypes = [P, I]
    L.cssg_system_lanes.argtypes = [P, P]
    L.cssg_system_set_lane_split.argtypes = [P, I]
    L.cssg_system_lane_split.argtypes = [P, P]
    L.cssg_system_source_costs.argtypes = [P, I, P]
    L.cssg_system_set_pass_groups.argtypes = [P, I, I]
    L.cssg_system_pass_groups.argtypes = [P, P, P]
    L.cssg_system_kernels_per_audit_step.argtypes = [P, P]
    L.cssg_system_screen_audit_status.argtypes = [P, P]
    L.cssg_screen_features.argtypes = [P, P, D, I, P, P, P, P, P, P]
    L.cssg_mlp_infer.argtypes = [P, P, I, P, P, P]
    L.cssg_mlp_grad.argtypes = [P, P, P, I, P, P, P]
    L.cssg_mlp_adam.argtypes = [P, P, P, P, P, I, ctypes.c_float, I]
    for name in EXPORTS:
        fn = getattr(L, name)
        if fn.restype is None and name not in ("cssg_last_error", "cssg_version", "cssg_ctx_stream"):
            fn.restype = I
    _lib = L
    return L


def check(rc: int, what: str = ""):
    if rc != CSSG_OK:
        msg = load().cssg_last_error().decode()
        raise CssgError(f"{what}: error {rc}: {msg}")
