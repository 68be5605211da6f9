"""kdgb -- GB300 kd-tree builder and ray tracer (host-side Python mirror).

The compute runs in libkdgb.so (hand-written sm_103a CUDA behind the C ABI in
include/kdgb.h).  This module is a thin host layer over that ABI with the
reference's plugin names:

* ``TriangleMap``  -- Utils/CUDA/TriangleMap.h:31-83 (Create, setters, GetNodes)
* ``RayTracer``, ``ShortStack``, ``BruteTracer`` -- the IRayTracer family
  (Utils/CUDA/IRayTracer.h:28-58); ``Trace`` returns first-hit buffers
  instead of drawing into an OpenGL canvas.
* ``KDTree`` -- the handle itself (build / rebuild / upload / view / trace).

PyTorch supplies device memory and the current stream; nothing here falls
back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import scenes
from ._lib import (BUILD_REFERENCE, BUILD_TUNED, ISECT_MOELLER, ISECT_WOOP, SCHEDULE_GRID, SCHEDULE_QUEUE, ERR_CAPACITY, ERR_INVALID_ARGUMENT, ERR_NO_DEVICE, FINF, LEAF, LOWER_BALANCED, LOWER_BITMAP, LOWER_SAH,
                   SPLIT_BOX, SPLIT_DIVIDE, SPLIT_SPLIT,
                   TIE_LOWEST_ID, TIE_REF_LAST, TRACER_BRUTE, TRACER_RESTART, TRACER_SHORTSTACK, X, Y, Z,
                   AutotuneResult, BuildParams, BuildStats, KdgbError, Light, light, PhotonParams, TraceParams, TreeView, build_params, check,
                   lib, library_path, photon_params, trace_params)

__all__ = ["KDTree", "Graph", "SmPartition", "autotune", "AutotuneResult", "Light", "light", "TriangleMap", "RayTracer", "ShortStack", "BruteTracer", "trace_brute", "build_params",
           "trace_params", "photon_params", "PhotonParams", "scenes", "KdgbError", "LEAF", "X", "Y", "Z", "LOWER_BITMAP", "LOWER_SAH",
           "LOWER_BALANCED", "SPLIT_BOX", "SPLIT_DIVIDE", "SPLIT_SPLIT",
           "BUILD_REFERENCE", "BUILD_TUNED", "TRACER_RESTART", "TRACER_SHORTSTACK", "TRACER_BRUTE",
           "TIE_LOWEST_ID", "TIE_REF_LAST", "ISECT_MOELLER", "ISECT_WOOP", "SCHEDULE_GRID", "SCHEDULE_QUEUE", "FINF",
           "lib", "library_path"]


def _torch():
    import torch
    return torch


def _stream(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _dev(a, dtype, shape_last=None):
    """A contiguous CUDA tensor of `dtype` from a tensor or numpy array."""
    torch = _torch()
    if isinstance(a, np.ndarray):
        a = torch.from_numpy(np.ascontiguousarray(a))
    if not a.is_cuda:
        a = a.cuda()
    a = a.to(dtype).contiguous()
    if shape_last is not None:
        a = a.reshape(-1, shape_last)
    return a


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else C.c_void_p(0)


@dataclass
class HostTree:
    """Tree arrays copied to host memory (KDNode / TriangleNode SoA)."""
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


class KDTree:
    """Owner of one kdgb_tree handle."""

    def __init__(self, handle: C.c_void_p, n_tris: int, stream: int = 0):
        self._h = handle
        self.n_tris = n_tris
        # The stream of the last call that queued work on this handle: the
        # handle's memory is freed ordered on it (kdgb_tree_release).
        self._last_stream = stream

    def _on(self, stream=None) -> C.c_void_p:
        """The raw stream of a call, remembered as the handle's last."""
        self._last_stream = _stream(stream)
        return C.c_void_p(self._last_stream)

    # -- construction -----------------------------------------------------
    @classmethod
    def build(cls, tris, params: BuildParams | None = None, stream=None, **kw) -> "KDTree":
        tri = _dev(tris, _torch().float32, 9)
        p = params if params is not None else build_params(**kw)
        h = C.c_void_p()
        st = _stream(stream)
        check(lib().kdgb_build(_ptr(tri), tri.shape[0], C.byref(p), C.byref(h), C.c_void_p(st)), "kdgb_build")
        return cls(h, tri.shape[0], st)

    def rebuild(self, tris, params: BuildParams | None = None, stream=None, **kw) -> None:
        tri = _dev(tris, _torch().float32, 9)
        p = params if params is not None else build_params(**kw)
        check(lib().kdgb_rebuild(self._h, _ptr(tri), tri.shape[0], C.byref(p), self._on(stream)), "kdgb_rebuild")
        self.n_tris = tri.shape[0]

    @classmethod
    def upload(cls, arrays, tris: np.ndarray, stream=None) -> "KDTree":
        """Creates a handle from host tree arrays (any object with the
        HostTree fields, e.g. a CPU-built tree) and host triangles."""
        tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
        keep = {}

        def host(name, dtype):
            a = np.ascontiguousarray(getattr(arrays, name), dtype=dtype)
            keep[name] = a
            return a.ctypes.data_as(C.c_void_p)

        v = TreeView()
        v.n_nodes = int(np.asarray(arrays.info).shape[0])
        v.n_refs = int(np.asarray(arrays.prim_indices).shape[0])
        v.n_upper_leaves = int(np.asarray(arrays.leaf_ids).shape[0])
        v.n_tris = tris.shape[0]
        v.info = host("info", np.int8)
        v.split = host("split", np.float32)
        v.aabb_min = host("aabb_min", np.float32)
        v.aabb_max = host("aabb_max", np.float32)
        v.prim_index = host("prim_index", np.int32)
        v.bitmap = host("bitmap", np.int32)
        v.children = host("children", np.int32)
        v.area = host("area", np.float32)
        v.parent = host("parent", np.int32)
        v.prim_indices = host("prim_indices", np.int32)
        v.leaf_ids = host("leaf_ids", np.int32)
        h = C.c_void_p()
        st = _stream(stream)
        check(lib().kdgb_tree_upload(C.byref(v), tris.ctypes.data_as(C.c_void_p), tris.shape[0], C.byref(h),
                                     C.c_void_p(st)), "kdgb_tree_upload")
        return cls(h, tris.shape[0], st)

    def close(self) -> None:
        """Frees the handle after the work queued on the stream it was last
        used on (kdgb_tree_release)."""
        if self._h:
            h, self._h = self._h, None
            check(lib().kdgb_tree_release(h, C.c_void_p(self._last_stream)), "kdgb_tree_release")

    def __del__(self):
        try:
            if self._h:
                h, self._h = self._h, None
                lib().kdgb_tree_release(h, C.c_void_p(self._last_stream))
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- inspection -------------------------------------------------------
    def view(self) -> TreeView:
        v = TreeView()
        check(lib().kdgb_tree_view_get(self._h, C.byref(v)), "kdgb_tree_view_get")
        return v

    def stats(self) -> BuildStats:
        s = BuildStats()
        check(lib().kdgb_tree_stats(self._h, C.byref(s)), "kdgb_tree_stats")
        return s

    def to_host(self) -> HostTree:
        """Copies the SoA tree arrays to host memory (kdgb_tree_download)."""
        v = self.view()
        n, r, nl = v.n_nodes, v.n_refs, v.n_upper_leaves
        h = HostTree(info=np.empty(n, np.int8), split=np.empty(n, np.float32),
                     aabb_min=np.empty((n, 4), np.float32), aabb_max=np.empty((n, 4), np.float32),
                     prim_index=np.empty(n, np.int32), bitmap=np.empty(n, np.int32),
                     children=np.empty((n, 2), np.int32), area=np.empty(n, np.float32),
                     parent=np.empty(n, np.int32), prim_indices=np.empty(r, np.int32),
                     leaf_ids=np.empty(nl, np.int32))
        dst = TreeView()
        for name in ("info", "split", "aabb_min", "aabb_max", "prim_index", "bitmap", "children", "area",
                     "parent", "prim_indices", "leaf_ids"):
            setattr(dst, name, getattr(h, name).ctypes.data_as(C.c_void_p))
        dst.n_nodes, dst.n_refs, dst.n_upper_leaves = n, r, nl
        check(lib().kdgb_tree_download(self._h, C.byref(dst)), "kdgb_tree_download")
        return h

    # -- tracing ----------------------------------------------------------
    def trace(self, o, d, params: TraceParams | None = None, stream=None, out=None, **kw):
        """First hit of each ray: (hit int32, t, u, v float32) CUDA tensors."""
        torch = _torch()
        o = _dev(o, torch.float32, 3)
        d = _dev(d, torch.float32, 3)
        n = o.shape[0]
        p = params if params is not None else trace_params(**kw)
        if out is None:
            out = (torch.empty(n, dtype=torch.int32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device))
        hit, t, u, v = out
        check(lib().kdgb_trace(self._h, C.byref(p), _ptr(o), _ptr(d), n, _ptr(hit), _ptr(t), _ptr(u), _ptr(v),
                               self._on(stream)), "kdgb_trace")
        return hit, t, u, v

    def trace_shadow(self, points, light, params: TraceParams | None = None, stream=None, **kw):
        torch = _torch()
        pts = _dev(points, torch.float32, 3)
        p = params if params is not None else trace_params(**kw)
        lp = (C.c_float * 3)(*[float(x) for x in light])
        occ = torch.empty(pts.shape[0], dtype=torch.int32, device=pts.device)
        check(lib().kdgb_trace_shadow(self._h, C.byref(p), _ptr(pts), pts.shape[0], lp, _ptr(occ),
                                      self._on(stream)), "kdgb_trace_shadow")
        return occ

    def trace_primary_shadow(self, o, d, light, params: TraceParams | None = None, stream=None, out=None, **kw):
        torch = _torch()
        o = _dev(o, torch.float32, 3)
        d = _dev(d, torch.float32, 3)
        n = o.shape[0]
        p = params if params is not None else trace_params(**kw)
        lp = (C.c_float * 3)(*[float(x) for x in light])
        if out is None:
            out = (torch.empty(n, dtype=torch.int32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.int32, device=o.device))
        hit, t, u, v, occ = out
        check(lib().kdgb_trace_primary_shadow(self._h, C.byref(p), _ptr(o), _ptr(d), n, lp, _ptr(hit), _ptr(t),
                                              _ptr(u), _ptr(v), _ptr(occ), self._on(stream)),
              "kdgb_trace_primary_shadow")
        return hit, t, u, v, occ

    def count_steps(self, o, d, light, params: TraceParams | None = None, stream=None, out=None, **kw):
        """trace_primary_shadow (short-stack) with traversal step counters
        (kdgb_trace_count_steps): returns the outputs and a dict of the
        primary and shadow rays' node records read, leaves reached, leaf
        boxes read and triangle records tested."""
        torch = _torch()
        o = _dev(o, torch.float32, 3)
        d = _dev(d, torch.float32, 3)
        n = o.shape[0]
        p = params if params is not None else trace_params(**kw)
        lp = (C.c_float * 3)(*[float(x) for x in light])
        if out is None:
            out = (torch.empty(n, dtype=torch.int32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.float32, device=o.device),
                   torch.empty(n, dtype=torch.int32, device=o.device))
        hit, t, u, v, occ = out
        counts = (C.c_uint64 * 8)()
        check(lib().kdgb_trace_count_steps(self._h, C.byref(p), _ptr(o), _ptr(d), n, lp, _ptr(hit), _ptr(t),
                                           _ptr(u), _ptr(v), _ptr(occ), counts, self._on(stream)),
              "kdgb_trace_count_steps")
        names = ("node", "leaf", "box", "tri")
        steps = {"primary": {k: int(counts[j]) for j, k in enumerate(names)},
                 "shadow": {k: int(counts[4 + j]) for j, k in enumerate(names)}}
        return (hit, t, u, v, occ), steps


def _trace_photons(self, n_photons: int, params: TraceParams | None = None, photons=None, stream=None, out=None,
                   **kw):
    """Photon segments: (hit int32, t float32) CUDA tensors of shape
    (n_photons, bounces + 1)."""
    torch = _torch()
    p = params if params is not None else trace_params(**kw)
    ph = photons if photons is not None else photon_params()
    S = ph.bounces + 1
    if out is None:
        out = (torch.empty((n_photons, S), dtype=torch.int32, device="cuda"),
               torch.empty((n_photons, S), dtype=torch.float32, device="cuda"))
    hit, t = out
    check(lib().kdgb_trace_photons(self._h, C.byref(p), C.byref(ph), n_photons, _ptr(hit), _ptr(t),
                                   self._on(stream)), "kdgb_trace_photons")
    return hit, t


KDTree.trace_photons = _trace_photons


def _trace_shaded(self, o, d, n0, n1, n2, c0, params: TraceParams | None = None, light_params: Light | None = None,
                  max_bounces: int = 0, stream=None, out=None, **kw):
    """Shaded pixels (kdgb_trace_shaded): (n, 4) uint8 CUDA tensor.  n0/n1/n2:
    (T, 4) float32 vertex normals per triangle, c0: (T, 4) uint8 colours."""
    torch = _torch()
    o = _dev(o, torch.float32, 3)
    d = _dev(d, torch.float32, 3)
    n0, n1, n2 = (_dev(x, torch.float32, 4) for x in (n0, n1, n2))
    c0 = _dev(c0, torch.uint8, 4)
    n = o.shape[0]
    p = params if params is not None else trace_params(**kw)
    L = light_params if light_params is not None else light()
    if out is None:
        out = torch.empty((n, 4), dtype=torch.uint8, device=o.device)
    check(lib().kdgb_trace_shaded(self._h, C.byref(p), _ptr(n0), _ptr(n1), _ptr(n2), _ptr(c0), C.byref(L),
                                  max_bounces, _ptr(o), _ptr(d), n, _ptr(out), self._on(stream)),
          "kdgb_trace_shaded")
    return out


KDTree.trace_shaded = _trace_shaded


def _build_batch(cls, tris, mesh_offsets, params: BuildParams | None = None, stream=None, **kw) -> "KDTree":
    """One forest over meshes stored back to back (kdgb_build_batch);
    mesh_offsets has n_meshes + 1 entries."""
    tri = _dev(tris, _torch().float32, 9)
    off = np.ascontiguousarray(mesh_offsets, dtype=np.int32)
    p = params if params is not None else build_params(**kw)
    h = C.c_void_p()
    st = _stream(stream)
    check(lib().kdgb_build_batch(_ptr(tri), off.ctypes.data_as(C.c_void_p), off.shape[0] - 1, C.byref(p),
                                 C.byref(h), C.c_void_p(st)), "kdgb_build_batch")
    tree = cls(h, tri.shape[0], st)
    tree.mesh_offsets = off
    return tree


def _trace_batch(self, o, d, ray_mesh=None, rays_per_mesh: int = 0, params: TraceParams | None = None, stream=None,
                 out=None, **kw):
    """Rays of a batch (kdgb_trace_batch): hit ids relative to each mesh."""
    torch = _torch()
    o = _dev(o, torch.float32, 3)
    d = _dev(d, torch.float32, 3)
    rm = _dev(ray_mesh, torch.int32).reshape(-1) if ray_mesh is not None else None
    n = o.shape[0]
    p = params if params is not None else trace_params(**kw)
    if out is None:
        out = (torch.empty(n, dtype=torch.int32, device=o.device), torch.empty(n, dtype=torch.float32, device=o.device),
               torch.empty(n, dtype=torch.float32, device=o.device), torch.empty(n, dtype=torch.float32, device=o.device))
    hit, t, u, v = out
    check(lib().kdgb_trace_batch(self._h, C.byref(p), _ptr(o), _ptr(d), _ptr(rm), rays_per_mesh, n, _ptr(hit),
                                 _ptr(t), _ptr(u), _ptr(v), self._on(stream)), "kdgb_trace_batch")
    return hit, t, u, v


def _rebuild_batch(self, tris, mesh_offsets, params: BuildParams | None = None, stream=None, **kw) -> None:
    """Rebuilds this handle as a batch (kdgb_rebuild_batch)."""
    tri = _dev(tris, _torch().float32, 9)
    off = np.ascontiguousarray(mesh_offsets, dtype=np.int32)
    p = params if params is not None else build_params(**kw)
    check(lib().kdgb_rebuild_batch(self._h, _ptr(tri), off.ctypes.data_as(C.c_void_p), off.shape[0] - 1,
                                   C.byref(p), self._on(stream)), "kdgb_rebuild_batch")
    self.n_tris = tri.shape[0]
    self.mesh_offsets = off


KDTree.build_batch = classmethod(_build_batch)
KDTree.rebuild_batch = _rebuild_batch
KDTree.trace_batch = _trace_batch


class Graph:
    """A rebuild of a tree (and optionally a trace) recorded as one CUDA
    graph (kdgb_graph_create).  The triangle, ray and output tensors are
    recorded by address: refill them in place, then launch()."""

    def __init__(self, tree: KDTree, tris, mesh_offsets=None, params: BuildParams | None = None,
                 headroom: float = 1.25, o=None, d=None, ray_mesh=None, rays_per_mesh: int = 0,
                 trace: TraceParams | None = None, out=None, stream=None, **kw):
        torch = _torch()
        self.tree = tree
        self.tris = _dev(tris, torch.float32, 9)
        off = None if mesh_offsets is None else np.ascontiguousarray(mesh_offsets, dtype=np.int32)
        n_meshes = 1 if off is None else off.shape[0] - 1
        p = params if params is not None else build_params(**kw)
        tp = trace if trace is not None else trace_params()
        self.o = self.d = self.ray_mesh = None
        self.out = None
        n = 0
        if o is not None:
            self.o = _dev(o, torch.float32, 3)
            self.d = _dev(d, torch.float32, 3)
            self.ray_mesh = _dev(ray_mesh, torch.int32).reshape(-1) if ray_mesh is not None else None
            n = self.o.shape[0]
            dev = self.o.device
            self.out = out if out is not None else (
                torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.float32, device=dev),
                torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.float32, device=dev))
        hit, t, u, v = self.out if self.out is not None else (None, None, None, None)
        g = C.c_void_p()
        check(lib().kdgb_graph_create(tree._h, _ptr(self.tris), self.tris.shape[0],
                                      off.ctypes.data_as(C.c_void_p) if off is not None else None, n_meshes,
                                      C.byref(p), headroom, C.byref(tp), _ptr(self.o), _ptr(self.d),
                                      _ptr(self.ray_mesh), rays_per_mesh, n, _ptr(hit), _ptr(t), _ptr(u), _ptr(v),
                                      C.byref(g), tree._on(stream)), "kdgb_graph_create")
        self._g = g

    def launch(self, stream=None) -> None:
        check(lib().kdgb_graph_launch(self._g, self.tree._on(stream)), "kdgb_graph_launch")

    def status(self, stream=None) -> int:
        """Synchronises and returns the last launch's build status (0 = ok)."""
        return lib().kdgb_graph_status(self._g, self.tree._on(stream))

    def close(self) -> None:
        if getattr(self, "_g", None):
            lib().kdgb_graph_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class SmPartition:
    """The device's SMs in two partitions (kdgb_sm_partition_create): the
    first with at least `sms` SMs, the second with the rest.  stream(which)
    gives a torch stream whose kernels run on that partition only; a Graph
    created with such a stream keeps its rebuild there wherever it is
    launched.  Close the partition after the graphs captured on its streams."""

    def __init__(self, sms: int):
        p = C.c_void_p()
        check(lib().kdgb_sm_partition_create(int(sms), C.byref(p)), "kdgb_sm_partition_create")
        self._p = p
        self._streams = []

    def sms(self, which: int) -> int:
        n = C.c_int32()
        check(lib().kdgb_sm_partition_sms(self._p, int(which), C.byref(n)), "kdgb_sm_partition_sms")
        return n.value

    def stream(self, which: int, priority: int = 0):
        torch = _torch()
        s = C.c_void_p()
        check(lib().kdgb_sm_partition_stream(self._p, int(which), int(priority), C.byref(s)),
              "kdgb_sm_partition_stream")
        st = torch.cuda.ExternalStream(s.value)
        self._streams.append(st)
        return st

    def close(self) -> None:
        if getattr(self, "_p", None):
            self._streams = []
            lib().kdgb_sm_partition_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def autotune(tris, o=None, d=None, mesh_offsets=None, ray_mesh=None, rays_per_mesh: int = 0,
             build: BuildParams | None = None, trace: TraceParams | None = None, builds_per_trace: float = 1.0,
             reps: int = 3, stream=None) -> AutotuneResult:
    """kdgb_autotune: the leaf threshold, SAH bins, short-stack depth and
    block size that minimise builds_per_trace * rebuild_ms + trace_ms."""
    torch = _torch()
    tri = _dev(tris, torch.float32, 9)
    off = None if mesh_offsets is None else np.ascontiguousarray(mesh_offsets, dtype=np.int32)
    n_meshes = 1 if off is None else off.shape[0] - 1
    od = _dev(o, torch.float32, 3) if o is not None else None
    dd = _dev(d, torch.float32, 3) if d is not None else None
    rm = _dev(ray_mesh, torch.int32).reshape(-1) if ray_mesh is not None else None
    n = od.shape[0] if od is not None else 0
    bp = build if build is not None else build_params()
    tp = trace if trace is not None else trace_params()
    res = AutotuneResult()
    check(lib().kdgb_autotune(_ptr(tri), tri.shape[0], off.ctypes.data_as(C.c_void_p) if off is not None else None,
                              n_meshes, _ptr(od), _ptr(dd), _ptr(rm), rays_per_mesh, n, C.byref(bp), C.byref(tp),
                              builds_per_trace, reps, C.byref(res), C.c_void_p(_stream(stream))), "kdgb_autotune")
    return res


def backward(vertices, indices, o, d, hit, dL_dt, dL_du, dL_dv, out=None, stream=None):
    """dL/dvertex (V, 3) float32 for an indexed mesh, reusing the forward's
    hit ids (kdgb_backward); `out` is accumulated into when given."""
    torch = _torch()
    verts = _dev(vertices, torch.float32, 3)
    idx = _dev(indices, torch.int32).reshape(-1)
    o = _dev(o, torch.float32, 3)
    d = _dev(d, torch.float32, 3)
    hit = _dev(hit, torch.int32).reshape(-1)
    gt = _dev(dL_dt, torch.float32).reshape(-1)
    gu = _dev(dL_du, torch.float32).reshape(-1)
    gv = _dev(dL_dv, torch.float32).reshape(-1)
    if out is None:
        out = torch.zeros_like(verts)
    check(lib().kdgb_backward(_ptr(verts), verts.shape[0], _ptr(idx), idx.numel() // 3, _ptr(o), _ptr(d),
                              o.shape[0], _ptr(hit), _ptr(gt), _ptr(gu), _ptr(gv), _ptr(out),
                              C.c_void_p(_stream(stream))), "kdgb_backward")
    return out


def trace_brute(tris, o, d, tie: int = TIE_LOWEST_ID, stream=None):
    """BruteTracer over device triangles, without a tree."""
    torch = _torch()
    tri = _dev(tris, torch.float32, 9)
    o = _dev(o, torch.float32, 3)
    d = _dev(d, torch.float32, 3)
    n = o.shape[0]
    hit = torch.empty(n, dtype=torch.int32, device=o.device)
    t = torch.empty(n, dtype=torch.float32, device=o.device)
    u = torch.empty_like(t)
    v = torch.empty_like(t)
    check(lib().kdgb_trace_brute(_ptr(tri), tri.shape[0], tie, _ptr(o), _ptr(d), n, _ptr(hit), _ptr(t), _ptr(u),
                                 _ptr(v), C.c_void_p(_stream(stream))), "kdgb_trace_brute")
    return hit, t, u, v


class TriangleMap:
    """Utils/CUDA/TriangleMap.h:31-83 over the C ABI.  The scene is a (T, 9)
    triangle array (the GeometryList the reference collects from the scene
    graph); Create() builds, the getters return the handle's arrays."""

    BITMAP, BALANCED, SAH = 0, 1, 2
    BOX, DIVIDE, SPLIT = 0, 1, 2

    def __init__(self, tris=None):
        self.geometry = tris
        self.params = build_params()
        self.tree: KDTree | None = None
        self.construction_time = 0.0

    def SetGeometry(self, tris) -> None:
        self.geometry = tris

    def Create(self) -> None:
        if self.tree is None:
            self.tree = KDTree.build(self.geometry, self.params)
        else:
            self.tree.rebuild(self.geometry, self.params)
        self.construction_time = self.tree.stats().build_ms

    _LOWER = {BITMAP: LOWER_BITMAP, BALANCED: LOWER_BALANCED, SAH: LOWER_SAH}

    def SetLowerAlgorithm(self, algo: int) -> None:
        self.params.lower = self._LOWER[algo]

    def GetLowerAlgorithm(self) -> int:
        return {v: k for k, v in self._LOWER.items()}[self.params.lower]

    def SplitEmptySpace(self, s: bool) -> None:
        self.params.split_empty_space = int(bool(s))

    def IsSplittingEmptySpace(self) -> bool:
        return bool(self.params.split_empty_space)

    def SetSplitMethod(self, m: int) -> None:
        # SPLIT is accepted here and refused by Create(), where the reference
        # throws NotImplemented (TriangleMapUpperCreator.cu:551-552).
        self.params.split_method = {self.BOX: SPLIT_BOX, self.DIVIDE: SPLIT_DIVIDE, self.SPLIT: SPLIT_SPLIT}[m]

    def GetSplitMethod(self) -> int:
        return int(self.params.split_method)

    def SetPropagateBoundingBox(self, p: bool) -> None:
        self.params.propagate_aabbs = int(bool(p))

    def GetPropagateBoundingBox(self) -> bool:
        return bool(self.params.propagate_aabbs)

    def SetTraversalCost(self, t: float) -> None:
        self.params.traversal_cost = float(t)

    def GetTraversalCost(self) -> float:
        return float(self.params.traversal_cost)

    @staticmethod
    def SetEmptySpaceThreshold(t: float) -> None:
        TriangleMap._threshold = float(t)

    def GetConstructionTime(self) -> float:
        return self.construction_time

    def GetNodes(self) -> TreeView:
        return self.tree.view()

    def GetPrimitiveIndices(self):
        return self.tree.view().prim_indices


class IRayTracer:
    """IRayTracer (IRayTracer.h:28-58).  Trace(o, d) returns (hit, t, u, v)."""

    MOELLER, WOOP = 0, 1
    _tracer = TRACER_RESTART

    def __init__(self, triangle_map: TriangleMap):
        self.map = triangle_map
        self.params = trace_params(tracer=self._tracer)
        self.render_time = 0.0

    def SetLeafSkipping(self, s: bool) -> None:
        self.params.leaf_skipping = int(bool(s))

    def GetLeafSkipping(self) -> bool:
        return bool(self.params.leaf_skipping)

    def SetIntersectionAlgorithm(self, a: int) -> None:
        self.params.intersection = ISECT_WOOP if a == self.WOOP else ISECT_MOELLER

    def GetIntersectionAlgorithm(self) -> int:
        return self.WOOP if self.params.intersection == ISECT_WOOP else self.MOELLER

    def GetRenderTime(self) -> float:
        return self.render_time

    def Trace(self, o, d, tile_width: int = 0):
        torch = _torch()
        p = TraceParams.from_buffer_copy(self.params)
        p.tile_width = tile_width
        if not self.map.GetPropagateBoundingBox():
            p.leaf_skipping = 0  # Raytracer.cu:313
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = self.map.tree.trace(o, d, p)
        e1.record()
        e1.synchronize()
        self.render_time = e0.elapsed_time(e1)
        return out

    def HostTrace(self, o, d):
        """Single-ray trace for debugging (the reference's HostTrace): runs
        the same device kernel on one ray and returns host values."""
        hit, t, u, v = self.map.tree.trace(np.asarray(o, np.float32).reshape(1, 3),
                                           np.asarray(d, np.float32).reshape(1, 3), self.params)
        return int(hit.cpu()[0]), float(t.cpu()[0]), float(u.cpu()[0]), float(v.cpu()[0])


class RayTracer(IRayTracer):
    _tracer = TRACER_RESTART


class ShortStack(IRayTracer):
    _tracer = TRACER_SHORTSTACK


class BruteTracer(IRayTracer):
    _tracer = TRACER_BRUTE
