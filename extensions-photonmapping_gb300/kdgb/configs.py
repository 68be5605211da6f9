"""Parameters of the measured workloads, shared by bench.py and the parity
tests so that both run exactly the same configuration.

  small     4096-triangle height field (64x32 grid), 256x256 pinhole rays,
            SAH Ct=1 Ci=1.5 leaf threshold 8, kd-restart and brute force
  frame     1,000,000-triangle clustered scene, 1920x1080 pinhole rays with
            one shadow ray per hit toward LIGHT, short-stack depth 8;
            median/empty-space splits on the top 8 levels, then SAH
  photons   262,144-triangle clustered scene, 16M photons from LIGHT,
            3 diffuse bounces, Russian roulette p = 0.7
  batched   512 clustered meshes, log-uniform 1k..200k triangles, 64k random
            rays per mesh
  adjoint   100k-triangle height field (316x158 grid), 512x512 rays
"""
from __future__ import annotations

import numpy as np

from . import scenes

# SAH lower phase of the small and frame configurations: traversal cost 1,
# intersection cost 1.5, nodes of <= 8 triangles stay leaves.
SAH = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
SAH_DESC = "reference upper (median + empty space to <32 refs) + SAH lower Ct=1 Ci=1.5 min_leaf=8"
# The frame's build: median/empty-space splits on the top 8 levels, binned
# SAH (32 bins) down to nodes of < 32 references, then the SAH lower phase.
TUNED = dict(SAH, mode=1, upper_levels=8, sah_bins=32)
TUNED_DESC = ("median + empty space on the top 8 levels, binned SAH (32 bins) below to <32 refs, "
              "then SAH lower Ct=1 Ci=1.5 min_leaf=8")

FRAME_TRIS = 1_000_000
FRAME_SEED = 2
WIDTH, HEIGHT = 1920, 1080
LIGHT = (0.5, 3.0, 0.5)
STACK_DEPTH = 8

PHOTON_TRIS = 262_144
PHOTONS = 16 << 20
PHOTON_SEED = 3
PHOTON_BOUNCES = 3
PHOTON_SURVIVAL = 0.7

BATCH_MESHES = 512
BATCH_LO, BATCH_HI = 1000, 200_000
BATCH_RAYS_PER_MESH = 65536
BATCH_SEED = 40


def frame_scene(tris: int = FRAME_TRIS, width: int = WIDTH, height: int = HEIGHT):
    """The frame's triangles (T, 9) and its pinhole rays (row-major pixels)."""
    t = scenes.clustered(tris, seed=FRAME_SEED)
    o, d = scenes.camera_rays(width, height)
    return t, o, d


def batch_sizes(n_meshes: int = BATCH_MESHES, lo: int = BATCH_LO, hi: int = BATCH_HI,
                seed: int = BATCH_SEED) -> np.ndarray:
    """Triangle counts log-uniform in [lo, hi]."""
    u = scenes.uniform(seed, n_meshes, 0)
    return np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * u).astype(np.int64)


def batch_scene(n_meshes: int = BATCH_MESHES, lo: int = BATCH_LO, hi: int = BATCH_HI,
                rays_per_mesh: int = BATCH_RAYS_PER_MESH, seed: int = BATCH_SEED):
    """Meshes of the batched workload (mesh m is a clustered scene with seed
    seed + 1 + m), their offsets (n_meshes + 1 int32) and rays_per_mesh
    random rays per mesh, mesh-major: origins on the mesh's bounding sphere,
    directions toward uniform points of its box."""
    sizes = batch_sizes(n_meshes, lo, hi, seed)
    meshes = [scenes.clustered(int(s), seed=seed + 1 + m) for m, s in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    o = np.empty((n_meshes * rays_per_mesh, 3), np.float32)
    d = np.empty_like(o)
    for m, t in enumerate(meshes):
        v = t.reshape(-1, 3)
        ro, rd = scenes.random_rays(rays_per_mesh, seed + 1000 + m, v.min(0), v.max(0))
        o[m * rays_per_mesh:(m + 1) * rays_per_mesh] = ro
        d[m * rays_per_mesh:(m + 1) * rays_per_mesh] = rd
    return meshes, off, o, d
