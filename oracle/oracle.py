"""ctypes front end of the CPU oracle (libkdgb_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py as the checker and the
timed CPU baseline.  The product library never imports this module.
Its intersection primitives, upper and lower creators, tracers, shading loop
and shadow rays are pinned bit for bit to the reference's own code, compiled
unmodified and run on the host (refpin_lib, ref_upper, ref_lower, ref_build,
refpin_trace_lib, ref_trace, ref_shadow; tests/test_refpin*.py; see
kdgb_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libkdgb_oracle.so")

LEAF, X, Y, Z = 0, 1, 2, 3
LOWER_BITMAP, LOWER_SAH, LOWER_BALANCED = 0, 1, 2
SPLIT_BOX, SPLIT_DIVIDE = 0, 1
TIE_LOWEST_ID, TIE_REF_LAST = 0, 1
TRACER_RESTART, TRACER_SHORTSTACK, TRACER_BRUTE = 0, 1, 2
ISECT_MOELLER, ISECT_WOOP = 0, 1
FINF = np.float32(2139095040.0)


class BuildParams(C.Structure):
    _fields_ = [("lower", C.c_int32), ("split_empty_space", C.c_int32),
                ("propagate_aabbs", C.c_int32), ("empty_space_threshold", C.c_float),
                ("traversal_cost", C.c_float), ("intersection_cost", C.c_float),
                ("min_leaf", C.c_int32), ("esc_zmax_as_x", C.c_int32),
                ("max_levels", C.c_int32), ("leaf_size", C.c_int32), ("mode", C.c_int32),
                ("upper_levels", C.c_int32), ("sah_bins", C.c_int32), ("split_method", C.c_int32)]


class TraceParams(C.Structure):
    _fields_ = [("tracer", C.c_int32), ("leaf_skipping", C.c_int32), ("tie", C.c_int32),
                ("stack_depth", C.c_int32), ("max_iterations", C.c_int32), ("intersection", C.c_int32)]


class _Tree(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_refs", C.c_int32), ("n_upper_leaves", C.c_int32),
                ("upper_levels", C.c_int32), ("lower_levels", C.c_int32),
                ("info", C.POINTER(C.c_int8)), ("split", C.POINTER(C.c_float)),
                ("aabb_min", C.POINTER(C.c_float)), ("aabb_max", C.POINTER(C.c_float)),
                ("prim_index", C.POINTER(C.c_int32)), ("bitmap", C.POINTER(C.c_int32)),
                ("children", C.POINTER(C.c_int32)), ("area", C.POINTER(C.c_float)),
                ("parent", C.POINTER(C.c_int32)), ("prim_indices", C.POINTER(C.c_int32)),
                ("leaf_ids", C.POINTER(C.c_int32)), ("prim_min", C.POINTER(C.c_float)),
                ("prim_max", C.POINTER(C.c_float))]


_lib = None


def build_library(force: bool = False) -> str:
    """Compiles libkdgb_oracle.so with the committed Makefile (rebuilt when
    the source changed or the library was built on another host arch)."""
    stamp = os.path.join(_HERE, ".host_arch")
    here = platform.machine()
    if not (os.path.exists(stamp) and open(stamp).read().strip() == here):
        force = True
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "kdgb_oracle.c"))):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
        with open(stamp, "w") as f:
            f.write(here + "\n")
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build_library()
        L = C.CDLL(_LIB_PATH)
        P = C.c_void_p
        L.or_build.argtypes = [P, C.c_int32, C.POINTER(BuildParams), C.POINTER(_Tree)]
        L.or_tree_free.argtypes = [C.POINTER(_Tree)]
        L.or_trace.argtypes = [C.POINTER(_Tree), P, C.c_int32, C.POINTER(TraceParams), P, P,
                               C.c_int32, P, P, P, P, C.c_int32]
        L.or_trace_brute.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P, P, C.c_int32, P, P, P, P, C.c_int32]
        L.or_trace_brute_f64.argtypes = [P, C.c_int32, P, P, C.c_int32, P, P, P, P, C.c_int32]
        L.or_trace_shadow.argtypes = [C.POINTER(_Tree), P, C.c_int32, C.c_int32, P, C.c_int32, P, P, C.c_int32]
        L.or_moeller_trumbore.argtypes = [P, P, P, P, P, C.c_float, P]
        L.or_error_string.restype = C.c_char_p
        L.or_build_params_default.argtypes = [C.POINTER(BuildParams)]
        L.or_trace_params_default.argtypes = [C.POINTER(TraceParams)]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().or_error_string(rc).decode())


def build_params(**kw) -> BuildParams:
    p = BuildParams()
    lib().or_build_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def trace_params(**kw) -> TraceParams:
    p = TraceParams()
    lib().or_trace_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@dataclass
class Tree:
    """Tree arrays in the reference's KDNode / TriangleNode SoA layout."""
    info: np.ndarray
    split: np.ndarray
    aabb_min: np.ndarray
    aabb_max: np.ndarray
    prim_index: np.ndarray
    bitmap: np.ndarray
    children: np.ndarray
    area: np.ndarray
    parent: np.ndarray
    prim_indices: np.ndarray
    leaf_ids: np.ndarray
    prim_min: np.ndarray
    prim_max: np.ndarray
    upper_levels: int = 0
    lower_levels: int = 0

    @property
    def n_nodes(self) -> int:
        return int(self.info.shape[0])

    def as_struct(self):
        s = _Tree()
        s.n_nodes = self.n_nodes
        s.n_refs = int(self.prim_indices.shape[0])
        s.n_upper_leaves = int(self.leaf_ids.shape[0])
        for name, ctype in [("info", C.c_int8), ("split", C.c_float), ("aabb_min", C.c_float),
                            ("aabb_max", C.c_float), ("prim_index", C.c_int32), ("bitmap", C.c_int32),
                            ("children", C.c_int32), ("area", C.c_float), ("parent", C.c_int32),
                            ("prim_indices", C.c_int32), ("leaf_ids", C.c_int32),
                            ("prim_min", C.c_float), ("prim_max", C.c_float)]:
            arr = getattr(self, name)
            setattr(s, name, arr.ctypes.data_as(C.POINTER(ctype)))
        return s


def _copy(ptr, n, dtype, shape=None):
    if n == 0:
        return np.zeros(shape if shape else (0,), dtype=dtype)
    buf = np.ctypeslib.as_array(ptr, shape=(n,)).copy().astype(dtype, copy=False)
    return buf.reshape(shape) if shape else buf


def build(tris: np.ndarray, params: BuildParams | None = None, **kw) -> Tree:
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    p = params if params is not None else build_params(**kw)
    t = _Tree()
    _check(lib().or_build(_ptr(tris), tris.shape[0], C.byref(p), C.byref(t)))
    try:
        n, r, lf = t.n_nodes, t.n_refs, t.n_upper_leaves
        out = Tree(info=_copy(t.info, n, np.int8), split=_copy(t.split, n, np.float32),
                   aabb_min=_copy(t.aabb_min, 4 * n, np.float32, (n, 4)),
                   aabb_max=_copy(t.aabb_max, 4 * n, np.float32, (n, 4)),
                   prim_index=_copy(t.prim_index, n, np.int32), bitmap=_copy(t.bitmap, n, np.int32),
                   children=_copy(t.children, 2 * n, np.int32, (n, 2)), area=_copy(t.area, n, np.float32),
                   parent=_copy(t.parent, n, np.int32), prim_indices=_copy(t.prim_indices, r, np.int32),
                   leaf_ids=_copy(t.leaf_ids, lf, np.int32),
                   prim_min=_copy(t.prim_min, 4 * r, np.float32, (r, 4)),
                   prim_max=_copy(t.prim_max, 4 * r, np.float32, (r, 4)),
                   upper_levels=t.upper_levels, lower_levels=t.lower_levels)
    finally:
        lib().or_tree_free(C.byref(t))
    return out


def _rays(o, d):
    o = np.ascontiguousarray(o, dtype=np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(d, dtype=np.float32).reshape(-1, 3)
    assert o.shape == d.shape
    return o, d


def trace(tree: Tree | None, tris: np.ndarray, o, d, params: TraceParams | None = None,
          threads: int = 0, **kw):
    """First-hit trace; returns (hit int32, t, u, v float32)."""
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    o, d = _rays(o, d)
    n = o.shape[0]
    p = params if params is not None else trace_params(**kw)
    hit = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    u = np.empty(n, np.float32)
    v = np.empty(n, np.float32)
    if p.tracer == TRACER_BRUTE:
        _check(lib().or_trace_brute(_ptr(tris), tris.shape[0], p.tie, p.intersection, _ptr(o), _ptr(d), n,
                                    _ptr(hit), _ptr(t), _ptr(u), _ptr(v), threads))
    else:
        s = tree.as_struct()
        _check(lib().or_trace(C.byref(s), _ptr(tris), tris.shape[0], C.byref(p), _ptr(o), _ptr(d), n,
                              _ptr(hit), _ptr(t), _ptr(u), _ptr(v), threads))
    return hit, t, u, v


def trace_brute_f64(tris, o, d, threads: int = 0):
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    o, d = _rays(o, d)
    n = o.shape[0]
    hit = np.empty(n, np.int32)
    t = np.empty(n, np.float64)
    u = np.empty(n, np.float64)
    v = np.empty(n, np.float64)
    _check(lib().or_trace_brute_f64(_ptr(tris), tris.shape[0], _ptr(o), _ptr(d), n,
                                    _ptr(hit), _ptr(t), _ptr(u), _ptr(v), threads))
    return hit, t, u, v


def trace_shadow(tree: Tree, tris, points, light, threads: int = 0, intersection: int = 0):
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    lp = np.ascontiguousarray(light, dtype=np.float32).reshape(3)
    occ = np.empty(pts.shape[0], np.int32)
    s = tree.as_struct()
    _check(lib().or_trace_shadow(C.byref(s), _ptr(tris), tris.shape[0], intersection, _ptr(pts), pts.shape[0],
                                 _ptr(lp), _ptr(occ), threads))
    return occ


class PhotonParams(C.Structure):
    _fields_ = [("light", C.c_float * 3), ("seed", C.c_uint64), ("bounces", C.c_int32), ("survival", C.c_float)]


def trace_photons(tree: Tree, tris, n: int, light=(0.5, 3.0, 0.5), seed: int = 3, bounces: int = 3,
                  survival: float = 0.7, threads: int = 0, **kw):
    """Photon segments (hit, t) of shape (n, bounces + 1)."""
    L = lib()
    L.or_trace_photons.argtypes = [C.POINTER(_Tree), C.c_void_p, C.c_int32, C.POINTER(TraceParams),
                                   C.POINTER(PhotonParams), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    p = trace_params(**kw)
    ph = PhotonParams()
    ph.light = (C.c_float * 3)(*[float(x) for x in light])
    ph.seed, ph.bounces, ph.survival = seed, bounces, survival
    hit = np.empty((n, bounces + 1), np.int32)
    t = np.empty((n, bounces + 1), np.float32)
    s = tree.as_struct()
    _check(L.or_trace_photons(C.byref(s), _ptr(tris), tris.shape[0], C.byref(p), C.byref(ph), n, _ptr(hit),
                              _ptr(t), threads))
    return hit, t


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("ambient", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3)]


def light(**kw) -> Light:
    L = Light()
    lib().or_light_default(C.byref(L))
    for k, v in kw.items():
        setattr(L, k, (C.c_float * 3)(*[float(x) for x in v]))
    return L


def trace_shaded(tree: Tree | None, tris, o, d, n0, n1, n2, c0, light_params: Light | None = None,
                 max_bounces: int = 64, threads: int = 0, **kw):
    """Shaded RGBA8 pixels (n, 4) uint8 (or_trace_shaded)."""
    L = lib()
    L.or_trace_shaded.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(TraceParams), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.POINTER(Light), C.c_int32, C.c_void_p, C.c_void_p,
                                  C.c_int32, C.c_void_p, C.c_int32]
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    o, d = _rays(o, d)
    n0, n1, n2 = (np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 4) for x in (n0, n1, n2))
    c0 = np.ascontiguousarray(c0, dtype=np.uint8).reshape(-1, 4)
    p = trace_params(**kw)
    lp = light_params if light_params is not None else light()
    out = np.empty((o.shape[0], 4), np.uint8)
    s = tree.as_struct() if tree is not None else None
    _check(L.or_trace_shaded(C.c_void_p(C.addressof(s)) if s is not None else None, _ptr(tris), tris.shape[0],
                             C.byref(p), _ptr(n0), _ptr(n1), _ptr(n2), _ptr(c0), C.byref(lp), max_bounces, _ptr(o),
                             _ptr(d), o.shape[0], _ptr(out), threads))
    return out


def kpow(x: float, y: float) -> float:
    """The specular power restated from series (or_kpow)."""
    L = lib()
    L.or_kpow.argtypes = [C.c_float, C.c_float]
    L.or_kpow.restype = C.c_float
    return float(L.or_kpow(x, y))


def philox4x32_10(ctr, key):
    L = lib()
    L.or_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    L.or_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def moeller_trumbore(v0, v1, v2, o, d, t_max=float(FINF)):
    arrs = [np.ascontiguousarray(x, dtype=np.float32).reshape(3) for x in (v0, v1, v2, o, d)]
    out = np.zeros(3, np.float32)
    hit = lib().or_moeller_trumbore(*[_ptr(a) for a in arrs], t_max, _ptr(out))
    return bool(hit), out


# ---------------------------------------------------------------------------
# Pin test: the oracle's single primitives and the reference's own
# header-only code compiled unmodified (oracle/refpin -> oracle/_ref).
# ---------------------------------------------------------------------------
_REFPIN_DIR = os.path.join(_HERE, "refpin")
_REFPIN_LIB = os.path.join(_HERE, "_ref", "librefpin.so")
_REFPIN_TRACE_LIB = os.path.join(_HERE, "_ref", "librefpin_trace.so")
_refpin_trace = None
_REFPIN_UPPER_LIB = os.path.join(_HERE, "_ref", "librefpin_upper.so")
_refpin_upper = None
_refpin = None


# Where the pin recipe reads the reference's sources (its REF).
REFERENCE_TREE = os.environ.get("KDGB_REFERENCE_TREE", "/root/reference")


def reference_tree_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_TREE, "Utils", "CUDA", "IRayTracer.h"))


def _make_pin(target: str, lib_path: str, jobs: int = 1) -> bool:
    """Builds one pin library with oracle/refpin/Makefile.  False where the
    reference tree is absent (nothing to pin against: callers skip); a
    recipe that fails with the tree present raises, so a broken pin build
    cannot turn the pin tests into skips."""
    if not reference_tree_available():
        return False
    r = subprocess.run(["make", "-s", f"-j{jobs}", "-C", _REFPIN_DIR, f"REF={REFERENCE_TREE}", target],
                       capture_output=True, text=True)
    if r.returncode != 0 or not os.path.exists(lib_path):
        raise RuntimeError(f"pin recipe failed for {target} (REF={REFERENCE_TREE}):\n{r.stdout}\n{r.stderr}")
    return True


def refpin_lib():
    """Loads oracle/_ref/librefpin.so, building it with the committed recipe
    first.  Returns None where the reference tree is not available, so
    callers can skip; raises when the tree is there and the recipe fails."""
    global _refpin
    if _refpin is not None:
        return _refpin
    if not _make_pin("../_ref/librefpin.so", _REFPIN_LIB):
        return None
    L = C.CDLL(_REFPIN_LIB)
    F = C.POINTER(C.c_float)
    L.ref_moeller_trumbore.argtypes = [F, F, F, C.c_float, F]
    L.ref_moeller_trumbore.restype = C.c_int
    L.ref_adjust_dir.argtypes = [F]
    L.ref_adjust_dir.restype = None
    L.ref_ray_box.argtypes = [F, F, F, F]
    L.ref_ray_box.restype = C.c_int
    L.ref_woop_rows.argtypes = [F, F]
    L.ref_woop_rows.restype = None
    L.ref_woop.argtypes = [F, F, F, C.c_float, F]
    L.ref_woop.restype = C.c_int
    L.ref_tri_box_step3.argtypes = [F, F, F]
    L.ref_tri_box_step3.restype = C.c_int
    _refpin = L
    return L


def refpin_upper_lib():
    """Loads oracle/_ref/librefpin_upper.so (the reference's upper-phase
    kernels run on the host), building it with the committed recipe first.
    Returns None where the reference tree is not available (raises when
    it is and the recipe fails)."""
    global _refpin_upper
    if _refpin_upper is not None:
        return _refpin_upper
    if not _make_pin("../_ref/librefpin_upper.so", _REFPIN_UPPER_LIB):
        return None
    L = C.CDLL(_REFPIN_UPPER_LIB)
    L.ref_upper.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int] + \
        [C.c_void_p] * 15
    L.ref_upper.restype = C.c_int
    _refpin_upper = L
    return L


def ref_upper(tris: np.ndarray, split_method: int = SPLIT_BOX, split_empty_space: bool = True,
              propagate_aabbs: bool = True, empty_space_threshold: float = 0.35):
    """The reference's own upper creator (TriangleMapUpperCreator.cu, its
    kernels run on the host by the pin library).  Returns a dict of the node
    arrays (`amount` holds the upper leaves' reference counts), the upper-leaf
    references (prim_min, prim_max, prim_indices), leaf_ids and the level
    count, or None when the pin library is not available."""
    L = refpin_upper_lib()
    if L is None:
        return None
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    T = tris.shape[0]
    cap_nodes, cap_refs, cap_leaves = 16 * T + 64, 8 * T + 64, 4 * T + 64
    out = {
        "info": np.zeros(cap_nodes, np.int8), "split": np.zeros(cap_nodes, np.float32),
        "aabb_min": np.zeros((cap_nodes, 4), np.float32), "aabb_max": np.zeros((cap_nodes, 4), np.float32),
        "prim_index": np.zeros(cap_nodes, np.int32), "amount": np.zeros(cap_nodes, np.int32),
        "children": np.zeros((cap_nodes, 2), np.int32), "parent": np.zeros(cap_nodes, np.int32),
        "prim_min": np.zeros((cap_refs, 4), np.float32), "prim_max": np.zeros((cap_refs, 4), np.float32),
        "prim_indices": np.zeros(cap_refs, np.int32), "leaf_ids": np.zeros(cap_leaves, np.int32),
    }
    n_refs, n_leaves, levels = C.c_int(0), C.c_int(0), C.c_int(0)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    n = L.ref_upper(int(split_method), int(split_empty_space), int(propagate_aabbs), float(empty_space_threshold),
                    P(tris), T, cap_nodes, cap_refs, cap_leaves, P(out["info"]), P(out["split"]), P(out["aabb_min"]),
                    P(out["aabb_max"]), P(out["prim_index"]), P(out["amount"]), P(out["children"]),
                    P(out["parent"]), P(out["prim_min"]), P(out["prim_max"]), P(out["prim_indices"]),
                    C.byref(n_refs), P(out["leaf_ids"]), C.byref(n_leaves), C.byref(levels))
    if n < 0:
        raise RuntimeError("ref_upper: capacity too small")
    res = {k: out[k][:n] for k in ("info", "split", "aabb_min", "aabb_max", "prim_index", "amount", "children",
                                    "parent")}
    for k in ("prim_min", "prim_max", "prim_indices"):
        res[k] = out[k][:n_refs.value]
    res["leaf_ids"] = out["leaf_ids"][:n_leaves.value]
    res["levels"] = levels.value
    return res


def ref_build(tris: np.ndarray, lower: int = LOWER_BITMAP, split_method: int = SPLIT_BOX,
              split_empty_space: bool = True, propagate_aabbs: bool = True, empty_space_threshold: float = 0.35,
              traversal_cost: float = 24.0):
    """The reference's whole build from its own kernels: ref_upper, then the
    BITMAP creator's leaf conversion (TriangleMapBitmapCreator.cu:22-34, two
    lines restated here: its kernel sits in a .cu whose host code does not
    compile) or the SAH / BALANCED creator (ref_lower).  Returns a Tree (area
    zero for BITMAP) and the lower level count, or None when a pin library is
    not available."""
    r = ref_upper(tris, split_method, split_empty_space, propagate_aabbs, empty_space_threshold)
    if r is None:
        return None
    info, bitmap, leaves = r["info"].copy(), r["amount"].copy(), r["leaf_ids"]
    info[leaves] = LEAF
    bitmap[leaves] = (np.left_shift(1, bitmap[leaves].astype(np.int64)) - 1).astype(np.int32)
    n = info.shape[0]
    tree = Tree(info=info, split=r["split"], aabb_min=r["aabb_min"], aabb_max=r["aabb_max"],
                prim_index=r["prim_index"], bitmap=bitmap, children=r["children"], area=np.zeros(n, np.float32),
                parent=r["parent"], prim_indices=r["prim_indices"], leaf_ids=leaves, prim_min=r["prim_min"],
                prim_max=r["prim_max"], upper_levels=r["levels"])
    if lower == LOWER_BITMAP:
        return tree, 0
    res = ref_lower(tris, tree, lower, traversal_cost, propagate_aabbs, max_nodes=64 * n + 64)
    if res is None:
        return None
    nodes, levels = res
    m = nodes["info"].shape[0]
    parent = np.zeros(m, np.int32)
    parent[:n] = tree.parent
    out = Tree(info=nodes["info"], split=nodes["split"], aabb_min=nodes["aabb_min"], aabb_max=nodes["aabb_max"],
               prim_index=nodes["prim_index"], bitmap=nodes["bitmap"], children=nodes["children"], area=nodes["area"],
               parent=parent, prim_indices=tree.prim_indices, leaf_ids=leaves, prim_min=tree.prim_min,
               prim_max=tree.prim_max, upper_levels=tree.upper_levels, lower_levels=levels)
    return out, levels


class RefTraceScene(C.Structure):
    """ref_trace_scene of oracle/refpin/refpin_trace.h."""
    _fields_ = [("n_nodes", C.c_int32), ("info", C.c_void_p), ("split", C.c_void_p), ("children", C.c_void_p),
                ("prim_index", C.c_void_p), ("bitmap", C.c_void_p), ("aabb_min", C.c_void_p),
                ("aabb_max", C.c_void_p), ("prim_indices", C.c_void_p), ("n_tris", C.c_int32),
                ("p0", C.c_void_p), ("p1", C.c_void_p), ("p2", C.c_void_p), ("n0", C.c_void_p),
                ("n1", C.c_void_p), ("n2", C.c_void_p), ("c0", C.c_void_p)]


def refpin_trace_lib():
    """Loads oracle/_ref/librefpin_trace.so (the reference's Raytracer.cu,
    ShortStack.cu and BruteTracer.cu compiled unmodified, their traversal
    functions called on the host), building it with the committed recipe
    first.  Returns None where the reference tree is not available (raises
    when it is and the recipe fails)."""
    global _refpin_trace
    if _refpin_trace is not None:
        return _refpin_trace
    if not _make_pin("../_ref/librefpin_trace.so", _REFPIN_TRACE_LIB, jobs=4):
        return None
    L = C.CDLL(_REFPIN_TRACE_LIB)
    P, I = C.c_void_p, C.c_int
    S = C.POINTER(RefTraceScene)
    for name in ("ref_restart_set_light", "ref_shortstack_set_light", "ref_brute_set_light"):
        getattr(L, name).argtypes = [P, P, P, P]
        getattr(L, name).restype = None
    L.ref_kdrestart.argtypes = [S, I, I, P, P, I, P, P, P]
    L.ref_kdrestart.restype = None
    L.ref_shortstack.argtypes = [S, I, I, P, P, I, P, P]
    L.ref_shortstack.restype = None
    L.ref_exhaustive.argtypes = [S, I, P, P, I, P]
    L.ref_exhaustive.restype = None
    L.ref_shadow.argtypes = [S, I, P, I, P, P]
    L.ref_shadow.restype = None
    L.ref_shortstack_depth.restype = I
    L.ref_brute_max_prims.restype = I
    L.ref_trace_set_pow.argtypes = [P]
    L.ref_trace_set_pow.restype = None
    _refpin_trace = L
    return L


def _f4(a, w):
    a = np.asarray(a, np.float32).reshape(-1, 3)
    return np.ascontiguousarray(np.concatenate([a, np.full((a.shape[0], 1), w, np.float32)], axis=1))


def ref_trace(tracer: int, tree: Tree | None, tris, o, d, n0, n1, n2, c0, light_params: Light | None = None,
              intersection: int = ISECT_MOELLER, leaf_skipping: bool = True, oracle_pow: bool = True):
    """The reference's own shaded tracers, ray by ray on the host
    (refpin_trace_lib): KDRestart (TRACER_RESTART), ShortStackTrace
    (TRACER_SHORTSTACK) or Exhaustive (TRACER_BRUTE).  With oracle_pow the
    specular power is the oracle's or_kpow (which the CUDA kernel computes
    too); without it the C library's powf, the reference's host path.
    Returns (rgba (n, 4) uint8, extra): extra is (first_prim, first_thit) for
    kd-restart, last_thit for the short stack and None for brute force."""
    L = refpin_trace_lib()
    if L is None:
        return None
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    keep = [_f4(tris[:, 0:3], 1.0), _f4(tris[:, 3:6], 1.0), _f4(tris[:, 6:9], 1.0)]
    keep += [np.ascontiguousarray(x, np.float32).reshape(-1, 4) for x in (n0, n1, n2)]
    keep.append(np.ascontiguousarray(c0, np.uint8).reshape(-1, 4))
    sc = RefTraceScene()
    sc.n_tris = tris.shape[0]
    sc.p0, sc.p1, sc.p2, sc.n0, sc.n1, sc.n2, sc.c0 = (k.ctypes.data for k in keep)
    if tree is not None:
        sc.n_nodes = tree.n_nodes
        for name in ("info", "split", "children", "prim_index", "bitmap", "aabb_min", "aabb_max",
                     "prim_indices"):
            arr = np.ascontiguousarray(getattr(tree, name))
            keep.append(arr)
            setattr(sc, name, arr.ctypes.data)
    lp = light_params if light_params is not None else light()
    args = [C.cast(lp.position, C.c_void_p), C.cast(lp.ambient, C.c_void_p), C.cast(lp.diffuse, C.c_void_p),
            C.cast(lp.specular, C.c_void_p)]
    L.ref_trace_set_pow(C.cast(lib().or_kpow, C.c_void_p) if oracle_pow else None)
    o4, d4 = _f4(o, 1.0), _f4(d, 0.0)
    n = o4.shape[0]
    rgba = np.zeros((n, 4), np.uint8)
    woop = int(intersection == ISECT_WOOP)
    if tracer == TRACER_RESTART:
        L.ref_restart_set_light(*args)
        prim = np.empty(n, np.int32)
        th = np.empty((n, 3), np.float32)
        L.ref_kdrestart(C.byref(sc), woop, int(leaf_skipping), o4.ctypes.data, d4.ctypes.data, n, rgba.ctypes.data,
                        prim.ctypes.data, th.ctypes.data)
        return rgba, (prim, th)
    if tracer == TRACER_SHORTSTACK:
        L.ref_shortstack_set_light(*args)
        th = np.empty((n, 3), np.float32)
        L.ref_shortstack(C.byref(sc), woop, int(leaf_skipping), o4.ctypes.data, d4.ctypes.data, n,
                         rgba.ctypes.data, th.ctypes.data)
        return rgba, th
    L.ref_brute_set_light(*args)
    L.ref_exhaustive(C.byref(sc), woop, o4.ctypes.data, d4.ctypes.data, n, rgba.ctypes.data)
    return rgba, None


def ref_shadow(tree: Tree, tris, points, light_pos, intersection: int = ISECT_MOELLER):
    """The reference's own ShadowRay (Raytracer.cu:108-163) per point: 1.0 lit,
    0.0 in shadow; None where the pin library is not available."""
    L = refpin_trace_lib()
    if L is None:
        return None
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    keep = [_f4(tris[:, 0:3], 1.0), _f4(tris[:, 3:6], 1.0), _f4(tris[:, 6:9], 1.0)]
    sc = RefTraceScene()
    sc.n_tris = tris.shape[0]
    sc.p0, sc.p1, sc.p2 = (k.ctypes.data for k in keep)
    sc.n_nodes = tree.n_nodes
    for name in ("info", "split", "children", "prim_index", "bitmap", "aabb_min", "aabb_max", "prim_indices"):
        arr = np.ascontiguousarray(getattr(tree, name))
        keep.append(arr)
        setattr(sc, name, arr.ctypes.data)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    lp = np.ascontiguousarray(light_pos, np.float32).reshape(3)
    lit = np.empty(pts.shape[0], np.float32)
    L.ref_shadow(C.byref(sc), int(intersection == ISECT_WOOP), pts.ctypes.data, pts.shape[0], lp.ctypes.data,
                 lit.ctypes.data)
    return lit


def pin_functions():
    """The oracle's counterparts of the reference's pinned primitives."""
    L = lib()
    F = C.POINTER(C.c_float)
    L.or_pin_adjust_dir.argtypes = [F]
    L.or_pin_adjust_dir.restype = None
    L.or_pin_ray_box.argtypes = [F, F, F, F]
    L.or_pin_ray_box.restype = C.c_int
    L.or_pin_woop_rows.argtypes = [F, F]
    L.or_pin_woop_rows.restype = None
    L.or_pin_woop.argtypes = [F, F, F, C.c_float, F]
    L.or_pin_woop.restype = C.c_int
    L.or_pin_tri_box.argtypes = [F, F, F]
    L.or_pin_tri_box.restype = C.c_int
    return L


def ref_lower(tris: np.ndarray, upper: Tree, lower: int, traversal_cost: float, propagate: bool = True,
              max_nodes: int | None = None):
    """The reference's own lower creator (SAH or BALANCED, its kernels run on
    the host by the pin library) over the upper phase of `upper`, a tree built
    with the BITMAP lower creator (its upper part is the same for every lower
    creator).  Returns the node arrays and the lower level count, or None when
    the pin library is not available."""
    L = refpin_lib()
    if L is None:
        return None
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    n0 = upper.n_nodes
    cap = max_nodes if max_nodes is not None else 64 * max(n0, 1)
    out = {
        "info": np.zeros(cap, np.int8), "split": np.zeros(cap, np.float32),
        "aabb_min": np.zeros((cap, 4), np.float32), "aabb_max": np.zeros((cap, 4), np.float32),
        "prim_index": np.zeros(cap, np.int32), "bitmap": np.zeros(cap, np.int32),
        "children": np.zeros((cap, 2), np.int32), "area": np.zeros(cap, np.float32),
    }
    for k, v in out.items():
        v[:n0] = getattr(upper, k)
    # The upper leaves hand their reference counts to the lower creator.
    leaves = upper.leaf_ids
    out["bitmap"][leaves] = [bin(int(np.uint32(b))).count("1") for b in upper.bitmap[leaves]]
    out["info"][leaves] = 0
    levels = C.c_int(0)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    L.ref_lower.restype = C.c_int
    n = L.ref_lower(C.c_int(lower), C.c_int(int(propagate)), C.c_float(traversal_cost), P(tris), C.c_int(tris.shape[0]),
                    C.c_int(n0), C.c_int(cap), P(out["info"]), P(out["split"]), P(out["aabb_min"]),
                    P(out["aabb_max"]), P(out["prim_index"]), P(out["bitmap"]), P(out["children"]), P(out["area"]),
                    P(np.ascontiguousarray(upper.prim_indices)), P(np.ascontiguousarray(upper.prim_min)),
                    P(np.ascontiguousarray(upper.prim_max)), C.c_int(upper.prim_indices.shape[0]),
                    P(np.ascontiguousarray(leaves)), C.c_int(leaves.shape[0]), C.byref(levels))
    if n < 0:
        raise RuntimeError("ref_lower: node capacity too small")
    return {k: v[:n] for k, v in out.items()}, levels.value
