"""ctypes binding of libkdgb.so (the C ABI declared in include/kdgb.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

LEAF, X, Y, Z = 0, 1, 2, 3
LOWER_BITMAP, LOWER_SAH, LOWER_BALANCED = 0, 1, 2
SPLIT_BOX, SPLIT_DIVIDE, SPLIT_SPLIT = 0, 1, 2
BUILD_REFERENCE, BUILD_TUNED = 0, 1
TRACER_RESTART, TRACER_SHORTSTACK, TRACER_BRUTE = 0, 1, 2
TIE_LOWEST_ID, TIE_REF_LAST = 0, 1
ISECT_MOELLER, ISECT_WOOP = 0, 1
SCHEDULE_GRID, SCHEDULE_QUEUE = 0, 1

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_CAPACITY = 4
ERR_DEGENERATE = 5
ERR_NONFINITE = 6
ERR_TIMEOUT = 7
ERR_UNSUPPORTED = 8
ERR_NO_DEVICE = 9

FINF = 2139095040.0


class BuildParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("lower", C.c_int32), ("split_empty_space", C.c_int32),
                ("propagate_aabbs", C.c_int32), ("empty_space_threshold", C.c_float),
                ("traversal_cost", C.c_float), ("intersection_cost", C.c_float), ("min_leaf", C.c_int32),
                ("esc_zmax_as_x", C.c_int32), ("max_levels", C.c_int32), ("leaf_size", C.c_int32),
                ("upper_levels", C.c_int32), ("sah_bins", C.c_int32), ("split_method", C.c_int32)]


class TraceParams(C.Structure):
    _fields_ = [("tracer", C.c_int32), ("leaf_skipping", C.c_int32), ("tie", C.c_int32),
                ("stack_depth", C.c_int32), ("max_iterations", C.c_int32), ("block_size", C.c_int32),
                ("tile_width", C.c_int32), ("intersection", C.c_int32), ("schedule", C.c_int32)]


class TreeView(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_refs", C.c_int32), ("n_upper_leaves", C.c_int32),
                ("n_tris", C.c_int32), ("info", C.c_void_p), ("split", C.c_void_p), ("aabb_min", C.c_void_p),
                ("aabb_max", C.c_void_p), ("prim_index", C.c_void_p), ("bitmap", C.c_void_p),
                ("children", C.c_void_p), ("area", C.c_void_p), ("parent", C.c_void_p),
                ("prim_indices", C.c_void_p), ("leaf_ids", C.c_void_p), ("p0", C.c_void_p), ("p1", C.c_void_p),
                ("p2", C.c_void_p)]


class PhotonParams(C.Structure):
    _fields_ = [("light", C.c_float * 3), ("seed", C.c_uint64), ("bounces", C.c_int32), ("survival", C.c_float)]


class AutotuneResult(C.Structure):
    _fields_ = [("build", BuildParams), ("trace", TraceParams), ("build_ms", C.c_float), ("trace_ms", C.c_float),
                ("baseline", C.c_float), ("objective", C.c_float), ("trials", C.c_int32)]


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("ambient", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3)]


class BuildStats(C.Structure):
    _fields_ = [("upper_levels", C.c_int32), ("lower_levels", C.c_int32), ("n_nodes", C.c_int32),
                ("n_refs", C.c_int32), ("n_leaves", C.c_int32), ("max_depth", C.c_int32),
                ("build_ms", C.c_float)]


# Every symbol include/kdgb.h declares, with its ctypes signature.
P = C.c_void_p
SIGNATURES = {
    "kdgb_abi_version": (C.c_int, []),
    "kdgb_status_string": (C.c_char_p, [C.c_int]),
    "kdgb_last_error": (C.c_char_p, []),
    "kdgb_launch_count": (C.c_int64, []),
    "kdgb_build_params_default": (None, [C.POINTER(BuildParams)]),
    "kdgb_trace_params_default": (None, [C.POINTER(TraceParams)]),
    "kdgb_build": (C.c_int, [P, C.c_int32, C.POINTER(BuildParams), C.POINTER(C.c_void_p), P]),
    "kdgb_rebuild": (C.c_int, [P, P, C.c_int32, C.POINTER(BuildParams), P]),
    "kdgb_tree_upload": (C.c_int, [C.POINTER(TreeView), P, C.c_int32, C.POINTER(C.c_void_p), P]),
    "kdgb_tree_destroy": (C.c_int, [P]),
    "kdgb_tree_release": (C.c_int, [P, P]),
    "kdgb_check_scan_giveup": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), P]),
    "kdgb_tree_view_get": (C.c_int, [P, C.POINTER(TreeView)]),
    "kdgb_tree_download": (C.c_int, [P, C.POINTER(TreeView)]),
    "kdgb_tree_stats": (C.c_int, [P, C.POINTER(BuildStats)]),
    "kdgb_trace": (C.c_int, [P, C.POINTER(TraceParams), P, P, C.c_int32, P, P, P, P, P]),
    "kdgb_trace_shadow": (C.c_int, [P, C.POINTER(TraceParams), P, C.c_int32, P, P, P]),
    "kdgb_trace_primary_shadow": (C.c_int, [P, C.POINTER(TraceParams), P, P, C.c_int32, P, P, P, P, P, P, P]),
    "kdgb_trace_count_steps": (C.c_int, [P, C.POINTER(TraceParams), P, P, C.c_int32, P, P, P, P, P, P,
                                         C.POINTER(C.c_uint64), P]),
    "kdgb_photon_params_default": (None, [C.POINTER(PhotonParams)]),
    "kdgb_trace_photons": (C.c_int, [P, C.POINTER(TraceParams), C.POINTER(PhotonParams), C.c_int32, P, P, P]),
    "kdgb_build_batch": (C.c_int, [P, P, C.c_int32, C.POINTER(BuildParams), C.POINTER(C.c_void_p), P]),
    "kdgb_rebuild_batch": (C.c_int, [P, P, P, C.c_int32, C.POINTER(BuildParams), P]),
    "kdgb_trace_batch": (C.c_int, [P, C.POINTER(TraceParams), P, P, P, C.c_int32, C.c_int32, P, P, P, P, P]),
    "kdgb_graph_create": (C.c_int, [P, P, C.c_int32, P, C.c_int32, C.POINTER(BuildParams), C.c_float,
                                    C.POINTER(TraceParams), P, P, P, C.c_int32, C.c_int32, P, P, P, P,
                                    C.POINTER(C.c_void_p), P]),
    "kdgb_graph_launch": (C.c_int, [P, P]),
    "kdgb_autotune": (C.c_int, [P, C.c_int32, P, C.c_int32, P, P, P, C.c_int32, C.c_int32, C.POINTER(BuildParams),
                                C.POINTER(TraceParams), C.c_float, C.c_int32, C.POINTER(AutotuneResult), P]),
    "kdgb_graph_status": (C.c_int, [P, P]),
    "kdgb_graph_destroy": (C.c_int, [P]),
    "kdgb_sm_partition_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "kdgb_sm_partition_sms": (C.c_int, [P, C.c_int32, C.POINTER(C.c_int32)]),
    "kdgb_sm_partition_stream": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "kdgb_sm_partition_destroy": (C.c_int, [P]),
    "kdgb_geometry_gather": (C.c_int, [P, C.c_int32, P, C.c_int32, P, P, P]),
    "kdgb_geometry_gather_attributes": (C.c_int, [P, P, C.c_int32, P, C.c_int32, P, P, P, P, P, P]),
    "kdgb_light_default": (None, [C.POINTER(Light)]),
    "kdgb_trace_shaded": (C.c_int, [P, C.POINTER(TraceParams), P, P, P, P, C.POINTER(Light), C.c_int32, P, P,
                                    C.c_int32, P, P]),
    "kdgb_trace_brute_shaded": (C.c_int, [P, C.c_int32, C.POINTER(TraceParams), P, P, P, P, C.POINTER(Light),
                                          C.c_int32, P, P, C.c_int32, P, P]),
    "kdgb_trace_brute_ex": (C.c_int, [P, C.c_int32, C.POINTER(TraceParams), P, P, C.c_int32, P, P, P, P, P]),
    "kdgb_osc_update_surface": (C.c_int, [P, P, C.c_int32, C.c_float, C.c_float, P]),
    "kdgb_backward": (C.c_int, [P, C.c_int32, P, C.c_int32, P, P, C.c_int32, P, P, P, P, P, P]),
    "kdgb_trace_brute": (C.c_int, [P, C.c_int32, C.c_int32, P, P, C.c_int32, P, P, P, P, P]),
    "kdgb_trace_brute_noalloc": (C.c_int, [P, C.c_int32, C.c_int32, P, P, C.c_int32, P, P, P, P, P]),
}

NOALLOC_MAX_TRIS = 65536  # KDGB_NOALLOC_MAX_TRIS

_lib = None


class KdgbError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        L = lib()
        msg = L.kdgb_status_string(status).decode()
        detail = L.kdgb_last_error().decode()
        super().__init__(f"{where}: {msg} ({detail})")


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    """The loaded libkdgb.so.  Raises when it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"libkdgb.so is not built ({path}); run __graft_entry__.build() first")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != OK:
        raise KdgbError(status, where)


def build_params(**kw) -> BuildParams:
    p = BuildParams()
    lib().kdgb_build_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def photon_params(**kw) -> PhotonParams:
    p = PhotonParams()
    lib().kdgb_photon_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "light":
            p.light = (C.c_float * 3)(*[float(x) for x in v])
        elif not hasattr(p, k):
            raise AttributeError(k)
        else:
            setattr(p, k, v)
    return p


def light(**kw) -> Light:
    L = Light()
    lib().kdgb_light_default(C.byref(L))
    for k, v in kw.items():
        if not hasattr(L, k):
            raise AttributeError(k)
        setattr(L, k, (C.c_float * 3)(*[float(x) for x in v]))
    return L


def trace_params(**kw) -> TraceParams:
    p = TraceParams()
    lib().kdgb_trace_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p
