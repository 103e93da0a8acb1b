"""ctypes binding of libnbody_gb300.so (the C ABI in include/nbody_gb300.h).

The library is built in-tree by ``nbody_gb300.build``.  There is no CPU
fallback: if the shared library is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnbody_gb300.so")

NBODY_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "capacity exceeded",
          5: "invalid state", 6: "no CUDA device", 7: "particle outside the root box"}

PREC_FP32, PREC_MIXED, PREC_FP64 = 0, 1, 2
INTEG_LEAPFROG, INTEG_EULER = 0, 1
DT_FIXED, DT_ADAPTIVE, DT_BLOCK = 0, 1, 2
ESCAPE_GROW, ESCAPE_ERROR = 0, 1

EXPORTS = ("nbody_default_params", "nbody_create", "nbody_destroy", "nbody_set_state", "nbody_get_state",
           "nbody_step", "nbody_compute_forces", "nbody_diagnostics", "nbody_tree_info", "nbody_get_tree",
           "nbody_get_interactions", "nbody_set_timing", "nbody_phase_times", "nbody_stream", "nbody_get_time",
           "nbody_last_error", "nbody_direct_forces", "nbody_get_stats", "nbody_flops_per_m2l", "nbody_flops_per_p2p",
           "nbody_measure_peaks", "nbody_direct_forces_static", "nbody_force_vjp", "nbody_forward_checkpointed",
           "nbody_backward", "nbody_device_memory", "nbody_trajectory_open", "nbody_trajectory_close",
           "nbody_set_timestep_control", "nbody_last_timestep", "nbody_set_escape_policy", "nbody_set_wait_limits",
           "nbody_selftest_wait", "nbody_forward_replay", "nbody_debug_bounds", "nbody_get_levels")


class Params(C.Structure):
    _fields_ = [("precision", C.c_int), ("order", C.c_int), ("leaf_capacity", C.c_int), ("max_level", C.c_int),
                ("theta", C.c_double), ("eps", C.c_double), ("G", C.c_double), ("dt", C.c_double),
                ("integrator", C.c_int), ("fixed_box", C.c_int), ("box_min", C.c_double * 3),
                ("box_size", C.c_double), ("device", C.c_int)]


class NbodyError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


_lib = None

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def load(path: str | None = None):
    """Loads the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("NBODY_LIB_PATH") or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m nbody_gb300.build`")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.nbody_default_params.argtypes = [C.POINTER(Params)]
    L.nbody_default_params.restype = None
    L.nbody_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.nbody_destroy.argtypes = [vp]
    L.nbody_set_state.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp]
    L.nbody_get_state.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp]
    L.nbody_direct_forces.argtypes = [vp, C.c_int64, vp, vp, vp]
    L.nbody_get_stats.argtypes = [vp, vp, C.c_int]
    L.nbody_flops_per_m2l.argtypes = [C.c_int]
    L.nbody_flops_per_m2l.restype = C.c_int64
    L.nbody_flops_per_p2p.argtypes = []
    L.nbody_flops_per_p2p.restype = C.c_int64
    L.nbody_measure_peaks.argtypes = [C.c_int, vp]
    L.nbody_direct_forces_static.argtypes = [C.c_int, C.c_int64, vp, vp, vp, C.c_double, C.c_double, C.c_int64, vp,
                                             vp, vp, vp]
    L.nbody_step.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
    L.nbody_force_vjp.argtypes = [vp, vp, vp, vp, vp]
    L.nbody_forward_checkpointed.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.nbody_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.nbody_device_memory.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.nbody_trajectory_open.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
    L.nbody_trajectory_close.argtypes = [vp]
    L.nbody_compute_forces.argtypes = [vp, vp, vp]
    L.nbody_diagnostics.argtypes = [vp, vp]
    L.nbody_tree_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int)]
    L.nbody_get_tree.argtypes = [vp, vp, vp, vp]
    L.nbody_get_interactions.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), vp]
    L.nbody_set_timing.argtypes = [vp, C.c_int]
    L.nbody_phase_times.argtypes = [vp, vp, C.c_int]
    L.nbody_stream.argtypes = [vp]
    L.nbody_stream.restype = vp
    L.nbody_get_time.argtypes = [vp, C.POINTER(C.c_double)]
    L.nbody_set_timestep_control.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
    L.nbody_last_timestep.argtypes = [vp, C.POINTER(C.c_double)]
    L.nbody_set_escape_policy.argtypes = [vp, C.c_int]
    L.nbody_set_wait_limits.argtypes = [vp, C.c_int64, C.c_int64]
    L.nbody_selftest_wait.argtypes = [vp, C.c_int]
    L.nbody_forward_replay.argtypes = [vp, vp, vp, vp, vp, C.c_int, vp, vp]
    L.nbody_debug_bounds.argtypes = []
    L.nbody_get_levels.argtypes = [vp, vp]
    L.nbody_last_error.argtypes = [vp]
    L.nbody_last_error.restype = C.c_char_p
    for name in EXPORTS:
        if name not in ("nbody_default_params", "nbody_stream", "nbody_last_error", "nbody_flops_per_m2l",
                        "nbody_flops_per_p2p"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(ctx, rc):
    if rc != NBODY_OK:
        msg = load().nbody_last_error(ctx)
        raise NbodyError(rc, msg.decode() if msg else "")


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
