"""Generates the golden fixtures in this directory from the CPU oracle.

The reference ships no tests or golden vectors and cannot be compiled here,
so these fixtures freeze the oracle's outputs (trees and first hits) on small
seeded inputs.  CPU tests check that the oracle still reproduces them and GPU
tests check the CUDA library against them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "extensions-photonmapping_gb300"))

import oracle as O  # noqa: E402
from kdgb import scenes  # noqa: E402

TREE_FIELDS = ("info", "split", "aabb_min", "aabb_max", "prim_index", "bitmap", "children", "area", "parent",
               "prim_indices", "leaf_ids")
SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
LIGHT = (0.5, 3.0, 0.5)


def cases():
    hf = scenes.heightfield(16, 8, seed=1)[0]
    o1, d1 = scenes.camera_rays(32, 32)
    cl = scenes.clustered(2000, seed=8)
    lo, hi = cl.reshape(-1, 3).min(0), cl.reshape(-1, 3).max(0)
    o2, d2 = scenes.random_rays(2048, 9, lo, hi)
    return {"heightfield_16x8": (hf, o1, d1), "clustered_2000": (cl, o2, d2)}


def make(name, tris, o, d):
    out = {"tris": tris, "ray_o": o, "ray_d": d}
    for tag, kw in (("bitmap", {}), ("sah", SAH_C1)):
        tree = O.build(tris, **kw)
        for f in TREE_FIELDS:
            out[f"{tag}_{f}"] = getattr(tree, f)
        for tracer, tname in ((O.TRACER_RESTART, "restart"), (O.TRACER_SHORTSTACK, "shortstack")):
            h, t, u, v = O.trace(tree, tris, o, d, tracer=tracer)
            out[f"{tag}_{tname}_hit"], out[f"{tag}_{tname}_t"] = h, t
            out[f"{tag}_{tname}_u"], out[f"{tag}_{tname}_v"] = u, v
        h, t, _, _ = O.trace(tree, tris, o, d, tracer=O.TRACER_RESTART, tie=O.TIE_REF_LAST)
        out[f"{tag}_restart_reflast_hit"] = h
        ph, pt = out[f"{tag}_restart_hit"], out[f"{tag}_restart_t"]
        pts = scenes.hit_points(o, d, pt, ph)
        out[f"{tag}_shadow_points"] = pts
        out[f"{tag}_shadow_occ"] = O.trace_shadow(tree, tris, pts, LIGHT)
    h, t, u, v = O.trace(None, tris, o, d, tracer=O.TRACER_BRUTE)
    out["brute_hit"], out["brute_t"], out["brute_u"], out["brute_v"] = h, t, u, v
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return out


if __name__ == "__main__":
    for name, (tris, o, d) in cases().items():
        make(name, tris, o, d)
        print("wrote", name)
