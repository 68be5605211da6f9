"""Seeded synthetic scenes and rays for the kd-tree build and trace path.

Every generator is deterministic for a given seed (SplitMix64 counter stream,
floats from the top 24 bits) and returns float32 arrays, so the same bytes can
be fed to the CUDA library and to the CPU oracle.  Geometry follows the
reference's own scene shapes where it has one:

* ``heightfield`` uses the quad -> two-triangle topology of
  Scene/OscCUDAMeshNode.cu:56-67 on a non-square grid, with heights
  z = 0.5 + sum of four seeded sinusoids of total amplitude 0.2.
* ``clustered`` builds the clustered test scene (Gaussian clusters of small
  triangles, two ground-plane triangles, long thin triangles).
* ``camera_rays`` is a pinhole camera whose pixel convention x/W*2-1 follows
  Utils/CUDA/IRayTracer.cu:62-65 (pixel corner, not centre).

Triangles are returned as ``(T, 9)`` float32: v0.xyz, v1.xyz, v2.xyz.
Rays are ``(n, 3)`` float32 origins and directions.
"""
from __future__ import annotations

import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n outputs of the SplitMix64 sequence for (seed, stream), counter based."""
    base = np.uint64((seed * 0x100000001B3 + stream * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        z = base + (np.arange(1, n + 1, dtype=np.uint64) * _GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """float64 uniforms in [0, 1) with 24-bit resolution."""
    z = splitmix64(seed, n, stream)
    return (z >> np.uint64(40)).astype(np.float64) * (1.0 / 16777216.0)


def normal(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """Standard normals by Box-Muller from two uniform streams."""
    u1 = uniform(seed, n, 2 * stream + 1)
    u2 = uniform(seed, n, 2 * stream + 2)
    u1 = np.maximum(u1, 1.0 / 16777216.0)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def grid_indices(nx: int, ny: int) -> np.ndarray:
    """Index buffer of an nx by ny quad grid, OscCUDAMeshNode.cu:56-67 order."""
    d = nx + 1
    m, n = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    m = m.reshape(-1).astype(np.int64)
    n = n.reshape(-1).astype(np.int64)
    idx = np.stack([m + n * d, m + (n + 1) * d, m + 1 + n * d,
                    m + 1 + n * d, m + (n + 1) * d, m + 1 + (n + 1) * d], axis=1)
    return idx.reshape(-1).astype(np.uint32)


def heightfield_vertices(nx: int, ny: int, seed: int, amplitude: float = 0.2) -> np.ndarray:
    """(nx+1)*(ny+1) vertices over [0,1]^2 with z = 0.5 + 4 seeded sinusoids."""
    r = uniform(seed, 12, stream=7)
    f = 1 + np.floor(r[0:4] * 4).astype(np.int64)
    g = 1 + np.floor(r[4:8] * 4).astype(np.int64)
    phi = r[8:12] * 2.0 * np.pi
    a = amplitude / 4.0
    i, j = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = i.reshape(-1) / nx
    y = j.reshape(-1) / ny
    z = np.full_like(x, 0.5)
    for k in range(4):
        z = z + a * np.sin(2.0 * np.pi * (f[k] * x + g[k] * y) + phi[k])
    return np.stack([x, y, z], axis=1).astype(np.float32)


def heightfield(nx: int, ny: int, seed: int = 1, amplitude: float = 0.2):
    """Height-field mesh: returns (tris (T,9) float32, vertices, indices)."""
    verts = heightfield_vertices(nx, ny, seed, amplitude)
    idx = grid_indices(nx, ny)
    tris = verts[idx.astype(np.int64)].reshape(-1, 9)
    return np.ascontiguousarray(tris, dtype=np.float32), verts, idx


def vertex_normals(verts: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """Per-vertex normals: the normalised sum of the adjacent faces' area
    weighted normals, as (V, 4) float32 with w = 0."""
    v = verts.astype(np.float64)
    t = idx.astype(np.int64).reshape(-1, 3)
    fn = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
    acc = np.zeros_like(v)
    for k in range(3):
        np.add.at(acc, t[:, k], fn)
    acc /= np.maximum(np.linalg.norm(acc, axis=1, keepdims=True), 1e-30)
    return np.concatenate([acc, np.zeros((v.shape[0], 1))], axis=1).astype(np.float32)


def shaded_box(nx: int = 32, ny: int = 16, seed: int = 1):
    """A height field inside four mirror-like walls, for the shading loop:
    returns (tris (T, 9), n0, n1, n2 (T, 4) float32 vertex normals per
    triangle, c0 (T, 4) uint8 colours).  The height field's colours are
    seeded with alphas of 255 (opaque), 128 and 0 (reflective), the walls
    have alpha 40, so rays take several bounces."""
    verts = heightfield_vertices(nx, ny, seed)
    idx = grid_indices(nx, ny).astype(np.int64)
    vn = vertex_normals(verts, idx)
    tris = verts[idx].reshape(-1, 9)
    nrm = vn[idx].reshape(-1, 3, 4)
    T = tris.shape[0]
    r = uniform(seed, 4 * T, stream=11).reshape(T, 4)
    c0 = np.floor(r * 256.0).clip(0, 255).astype(np.uint8)
    c0[:, 3] = np.array([255, 128, 0], np.uint8)[np.floor(r[:, 3] * 3).astype(np.int64).clip(0, 2)]
    lo, hi, top = -0.1, 1.1, 1.5
    corners = {"x0": [(lo, lo, 0), (lo, hi, 0), (lo, hi, top), (lo, lo, top)],
               "x1": [(hi, lo, 0), (hi, lo, top), (hi, hi, top), (hi, hi, 0)],
               "y0": [(lo, lo, 0), (lo, lo, top), (hi, lo, top), (hi, lo, 0)],
               "y1": [(lo, hi, 0), (hi, hi, 0), (hi, hi, top), (lo, hi, top)]}
    inward = {"x0": (1, 0, 0), "x1": (-1, 0, 0), "y0": (0, 1, 0), "y1": (0, -1, 0)}
    wt, wn, wc = [], [], []
    for k, q in corners.items():
        a, b, c, d = (np.array(p, np.float32) for p in q)
        n4 = np.array(inward[k] + (0,), np.float32)
        for tri in ((a, b, c), (a, c, d)):
            wt.append(np.concatenate(tri))
            wn.append(np.stack([n4, n4, n4]))
            wc.append(np.array([200, 210, 230, 40], np.uint8))
    tris = np.concatenate([tris, np.array(wt, np.float32)])
    nrm = np.concatenate([nrm, np.array(wn, np.float32)])
    c0 = np.concatenate([c0, np.array(wc, np.uint8)])
    n0, n1, n2 = (np.ascontiguousarray(nrm[:, k]) for k in range(3))
    return np.ascontiguousarray(tris, dtype=np.float32), n0, n1, n2, np.ascontiguousarray(c0)


def _frames(seed: int, n: int, stream: int):
    """Random orthonormal pairs (u, w) spanning a uniformly oriented plane."""
    nz = normal(seed, n, stream)
    ny = normal(seed, n, stream + 1)
    nxx = normal(seed, n, stream + 2)
    nrm = np.stack([nxx, ny, nz], axis=1)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-12)
    helper = np.where(np.abs(nrm[:, :1]) < 0.9, np.array([[1.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]]))
    u = np.cross(nrm, helper)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(nrm, u)
    return u, w


def clustered(T: int, seed: int = 2, clusters: int = 64, sigma: float = 0.02,
              thin: int | None = None) -> np.ndarray:
    """Clustered scene of T triangles: 2 ground-plane triangles over [-1,2]^2
    at z=0, `thin` long thin triangles (aspect 100:1, default 2000 or T/500
    for small T) and Gaussian clusters of small triangles (edge ~U(.001,.005))."""
    if thin is None:
        thin = min(2000, max(0, T // 500))
    ground = 2 if T >= 2 else T
    thin = max(0, min(thin, T - ground))
    n_cl = T - ground - thin
    out = np.empty((T, 9), dtype=np.float64)
    k = 0
    if ground == 2:
        out[0] = [-1, -1, 0, 2, -1, 0, -1, 2, 0]
        out[1] = [2, -1, 0, 2, 2, 0, -1, 2, 0]
        k = 2
    elif ground == 1:
        out[0] = [-1, -1, 0, 2, -1, 0, -1, 2, 0]
        k = 1
    if thin > 0:
        c = np.stack([uniform(seed, thin, 20 + a) for a in range(3)], axis=1)
        length = 0.05 + 0.15 * uniform(seed, thin, 23)
        u, w = _frames(seed, thin, 24)
        half = 0.5 * length[:, None]
        wid = (length / 100.0)[:, None]
        v0 = c - half * u
        v1 = c + half * u
        v2 = c + wid * w
        out[k:k + thin] = np.concatenate([v0, v1, v2], axis=1)
        k += thin
    if n_cl > 0:
        centers = np.stack([uniform(seed, clusters, 40 + a) for a in range(3)], axis=1)
        counts = np.full(clusters, n_cl // clusters, dtype=np.int64)
        counts[: n_cl % clusters] += 1
        owner = np.repeat(np.arange(clusters), counts)
        cen = centers[owner] + sigma * np.stack([normal(seed, n_cl, 50 + 3 * a) for a in range(3)], axis=1)
        edge = 0.001 + 0.004 * uniform(seed, n_cl, 60)
        u, w = _frames(seed, n_cl, 61)
        th0 = 2.0 * np.pi * uniform(seed, n_cl, 70)
        rad = (edge / math.sqrt(3.0))[:, None]
        vs = []
        for j in range(3):
            ang = (th0 + j * 2.0 * np.pi / 3.0)[:, None]
            vs.append(cen + rad * (np.cos(ang) * u + np.sin(ang) * w))
        out[k:] = np.concatenate(vs, axis=1)
    return np.ascontiguousarray(out.astype(np.float32))


def look_at_basis(eye, target, up):
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, dtype=np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    return eye, fwd, right, upv


def camera_rays(width: int, height: int, eye=(0.5, 0.5, 2.0), target=(0.0, 0.0, 0.0),
                up=(0.0, 1.0, 0.0), fov_deg: float = 60.0):
    """Pinhole primary rays in row-major pixel order (id = x + y*width).
    Pixel (x, y) maps to screen (x/W*2-1, y/H*2-1) as in IRayTracer.cu:62-65;
    directions are normalised in float64 and rounded to float32."""
    eye, fwd, right, upv = look_at_basis(eye, target, up)
    th = math.tan(math.radians(fov_deg) * 0.5)
    aspect = width / height
    x = np.arange(width, dtype=np.float64)
    y = np.arange(height, dtype=np.float64)
    sx = (x / width) * 2.0 - 1.0
    sy = (y / height) * 2.0 - 1.0
    SX, SY = np.meshgrid(sx, sy, indexing="xy")
    d = (fwd[None, None, :] + (SX[..., None] * th * aspect) * right[None, None, :]
         + (SY[..., None] * th) * upv[None, None, :])
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    d = d.reshape(-1, 3).astype(np.float32)
    o = np.broadcast_to(eye.astype(np.float32), d.shape).copy()
    return np.ascontiguousarray(o), np.ascontiguousarray(d)


def random_rays(n: int, seed: int, lo, hi):
    """Rays with origins uniform on the bounding sphere of box [lo, hi] and
    directions toward a uniform point inside the box (normalised)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    c = 0.5 * (lo + hi)
    r = 0.5 * np.linalg.norm(hi - lo) * 1.01 + 1e-6
    g = np.stack([normal(seed, n, 80 + 3 * a) for a in range(3)], axis=1)
    g /= np.maximum(np.linalg.norm(g, axis=1, keepdims=True), 1e-12)
    o = c + r * g
    p = lo + (hi - lo) * np.stack([uniform(seed, n, 90 + a) for a in range(3)], axis=1)
    d = p - o
    d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
    return (np.ascontiguousarray(o.astype(np.float32)), np.ascontiguousarray(d.astype(np.float32)))


def hit_points(o: np.ndarray, d: np.ndarray, t: np.ndarray, hit: np.ndarray) -> np.ndarray:
    """Hit points p = o + t*d in float32 with separately rounded multiply and
    add (the order the fused CUDA primary+shadow kernel uses)."""
    tt = np.where(hit >= 0, t, 0.0).astype(np.float32)
    m = (tt[:, None] * d).astype(np.float32)
    return np.ascontiguousarray((o + m).astype(np.float32))
