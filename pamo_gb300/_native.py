"""ctypes binding of the C ABI in include/pamo_gb300.h (the in-tree libpamo_gb300.so).

There is no fallback: when the library is missing or cannot be loaded every entry point raises.
"""

from __future__ import annotations

import ctypes
import os

from . import _build

PAMO_OK = 0
STATUS_NAMES = {
    0: "ok",
    1: "invalid argument",
    2: "out of device memory",
    3: "capacity exceeded",
    4: "iteration limit",
    5: "CUDA error",
    6: "invalid call order",
}

# every exported symbol of include/pamo_gb300.h with (restype, argtypes)
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_F32 = ctypes.c_float
_F64 = ctypes.c_double
_PI32 = ctypes.POINTER(ctypes.c_int32)
_PI64 = ctypes.POINTER(ctypes.c_int64)

SIGNATURES = {
    "pamo_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "pamo_ctx_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    "pamo_ctx_destroy": (ctypes.c_int, [_P]),
    "pamo_ctx_last_error": (ctypes.c_char_p, [_P]),
    "pamo_ctx_reset": (ctypes.c_int, [_P, _P]),
    "pamo_ctx_device_bytes": (ctypes.c_int64, [_P]),
    "pamo_ctx_set_option": (ctypes.c_int, [_P, ctypes.c_char_p, _I64]),
    "pamo_forward_round": (ctypes.c_int, [_P, _P, _P, _P, _I32, _I32, _I32, _F32, _F32, _I32, _I32, _P]),
    "pamo_legacy_round": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _F32, _F32, _I32, _P]),
    "pamo_point_mesh_sqdist": (ctypes.c_int, [_P, _I32, _P, _I32, _P, _I32, _P, _P, _P]),
    "pamo_face_min_angles": (ctypes.c_int, [_P, _P, _I32, _P, _P, _P]),
    "pamo_remesher_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), _I32]),
    "pamo_remesher_destroy": (ctypes.c_int, [_P]),
    "pamo_remesh": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _I32, _P, ctypes.POINTER(ctypes.c_int32),
                                   ctypes.POINTER(ctypes.c_int32), _P]),
    "pamo_remesh_result": (ctypes.c_int, [_P, _P, _P, _P]),
    "pamo_simplify_device_target": (ctypes.c_int, [_P, _P, _P, _I32, _I32, ctypes.c_int64, _I32, _F32, _I32, _I32,
                                                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                                   ctypes.POINTER(ctypes.c_int32), _P]),
    "pamo_tris_mean": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _P, _P]),
    "pamo_cost_probe": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _F32, _F32, _I32, _P, _P, _P, _I32, _PI32, _P]),
    "pamo_round_sizes": (ctypes.c_int, [_P, _PI32, _PI32, _PI32]),
    "pamo_round_outputs": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "pamo_round_stats": (ctypes.c_int, [_P, _PI64, _I32]),
    "pamo_simplify_device": (
        ctypes.c_int,
        [_P, _P, _P, _I32, _I32, _F64, _I32, _F32, _I32, _I64, _PI32, _PI32, _PI32, _P],
    ),
    "pamo_simplify": (ctypes.c_int, [_P, _P, _P, _P, _P, _F32]),
    "pamo_simplify_result": (ctypes.c_int, [_P, _P, _P, _P]),
    "pamo_simplify_round_faces": (ctypes.c_int, [_P, _PI32, _I32]),
    "pamo_simplify_round_ms": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _I32]),
    "pamo_kernel_time": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64), _I32]),
    "pamo_simplify_round_gpu_ms": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _I32]),
    "pamo_self_intersect": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _P, _P]),
    "pamo_self_intersect_noalloc": (ctypes.c_int, [_P, _P, _I32, _I32, _P, _P]),
    "pamo_server_submit_ex": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _F64, _I32, _F32, _I32, _PI64]),
    "pamo_server_fetch_f64": (ctypes.c_int, [_P, _I64, _P, _P]),
    "pamo_csr_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    "pamo_csr_destroy": (ctypes.c_int, [_P]),
    "pamo_csr_last_error": (ctypes.c_char_p, [_P]),
    "pamo_csr_set_option": (ctypes.c_int, [_P, ctypes.c_char_p, _I64]),
    "pamo_csr_simplify": (ctypes.c_int, [_P, _P, _P, _P, _P, _I32, _P, _I32, _F32, _I32, _I64, _P, _P, _P, _P, _P]),
    "pamo_csr_rounds": (ctypes.c_int, [_P, _PI32, _I32]),
    "pamo_run_totals": (ctypes.c_int, [_P, _PI64, _I32]),
    "pamo_launch_count": (ctypes.c_int64, []),
    "pamo_profile_enable": (ctypes.c_int, [_P, _I32]),
    "pamo_profile_read": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _PI64, _I32]),
    "pamo_batch_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, _I32]),
    "pamo_batch_destroy": (ctypes.c_int, [_P]),
    "pamo_batch_last_error": (ctypes.c_char_p, [_P]),
    "pamo_batch_simplify": (ctypes.c_int, [_P, _P, _P, _P, _P, _I32, _P, _I32, _F32, _I32, _I64, _P, _P, _P, _P, _P]),
    "pamo_batch_rounds": (ctypes.c_int, [_P, _PI32, _I32]),
    "pamo_server_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, _I32, _I64]),
    "pamo_server_destroy": (ctypes.c_int, [_P]),
    "pamo_server_last_error": (ctypes.c_char_p, [_P]),
    "pamo_server_submit": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _F64, _I32, _F32, _PI64]),
    "pamo_server_wait": (ctypes.c_int, [_P, _I32, _PI64, _PI32, _PI32, _PI32, ctypes.POINTER(ctypes.c_double)]),
    "pamo_server_fetch": (ctypes.c_int, [_P, _I64, _P, _P]),
    "pamo_server_stats": (ctypes.c_int, [_P, _PI64, _I32]),
    "pamo_server_job_bytes": (ctypes.c_int64, [_I32, _I32]),
    "pamo_mesh_process": (ctypes.c_int, [_P, _I32, _P, _I32, _P, _PI32, _P, _PI32]),
    "pamo_stage3_topology": (ctypes.c_int, [_P, _I32, _I32, _P, _PI32, _P, _I32, _PI32]),
    "pamo_stage3_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    "pamo_stage3_destroy": (ctypes.c_int, [_P]),
    "pamo_stage3_last_error": (ctypes.c_char_p, [_P]),
    "pamo_stage3_set_param": (ctypes.c_int, [_P, ctypes.c_char_p, _F64]),
    "pamo_safe_project": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _P, _P, _I32, _I32, _I32, _P, _P]),
    "pamo_stage3_stats": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _I32]),
}

STAGE3_STATS = ["particles", "triangles", "edges", "hinges", "steps", "newton_iters", "max_contacts",
                "radius_halvings", "do_nothing", "energy", "total_contacts", "candidate_rebuilds", "barrier_reruns"]

RUN_TOTALS = ["vertices", "faces", "edges", "winners", "query_tests", "pairs", "exact_pairs", "checks", "live_indexed",
              "collapsed"]

PHASES = ["load", "adjacency", "quadrics", "edge_cost", "collapse", "marks", "bvh_build", "bvh_query", "undo",
          "compact", "center"]

_LIB = None


class PamoError(RuntimeError):
    """A pamo_* call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"pamo: {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def lib_path() -> str:
    return _build.lib_path()


def load() -> ctypes.CDLL:
    """Load libpamo_gb300.so (raises when it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"pamo_gb300 CUDA library not found at {path}; build it with "
            "`python -c 'import pamo_gb300._build as b; b.build()'` (requires nvcc)"
        )
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int, ctx=None) -> None:
    if status != PAMO_OK:
        msg = ""
        if ctx is not None:
            raw = load().pamo_ctx_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise PamoError(status, msg)
