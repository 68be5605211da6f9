"""Golden fixtures (tests/golden/*.npz, made by make_golden.py from the oracle):
the oracle must keep reproducing them (CPU) and the CUDA library must match
them bit for bit (GPU)."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
LIGHT = (0.5, 3.0, 0.5)
TREE_FIELDS = ("info", "split", "aabb_min", "aabb_max", "prim_index", "bitmap", "children", "area", "parent",
               "prim_indices", "leaf_ids")


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)


def test_fixtures_present():
    assert len(FIXTURES) >= 2


@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_oracle_reproduces_golden(oracle, path):
    g = np.load(path)
    tris, o, d = g["tris"], g["ray_o"], g["ray_d"]
    for tag, kw in (("bitmap", {}), ("sah", SAH_C1)):
        tree = oracle.build(tris, **kw)
        for f in TREE_FIELDS:
            assert same(getattr(tree, f), g[f"{tag}_{f}"]), f"{tag} {f}"
        for tracer, tname in ((0, "restart"), (1, "shortstack")):
            h, t, u, v = oracle.trace(tree, tris, o, d, tracer=tracer)
            for k, arr in zip("htuv", (h, t, u, v)):
                key = f"{tag}_{tname}_" + {"h": "hit", "t": "t", "u": "u", "v": "v"}[k]
                assert same(arr, g[key]), key
        assert same(oracle.trace(tree, tris, o, d, tracer=0, tie=1)[0], g[f"{tag}_restart_reflast_hit"])
        assert same(oracle.trace_shadow(tree, tris, g[f"{tag}_shadow_points"], LIGHT), g[f"{tag}_shadow_occ"])
    h, t, u, v = oracle.trace(None, tris, o, d, tracer=2)
    assert same(h, g["brute_hit"]) and same(t, g["brute_t"]) and same(u, g["brute_u"]) and same(v, g["brute_v"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_cuda_matches_golden(kdgb_lib, cuda, path):
    g = np.load(path)
    tris, o, d = g["tris"], g["ray_o"], g["ray_d"]
    for tag, kw in (("bitmap", {}), ("sah", SAH_C1)):
        with kdgb_lib.KDTree.build(tris, **kw) as tree:
            host = tree.to_host()
            for f in TREE_FIELDS:
                assert same(getattr(host, f), g[f"{tag}_{f}"]), f"{tag} {f}"
            for tracer, tname in ((0, "restart"), (1, "shortstack")):
                h, t, u, v = (x.cpu().numpy() for x in tree.trace(o, d, tracer=tracer))
                assert same(h, g[f"{tag}_{tname}_hit"]) and same(t, g[f"{tag}_{tname}_t"])
                assert same(u, g[f"{tag}_{tname}_u"]) and same(v, g[f"{tag}_{tname}_v"])
            h = tree.trace(o, d, tracer=0, tie=1)[0].cpu().numpy()
            assert same(h, g[f"{tag}_restart_reflast_hit"])
            occ = tree.trace_shadow(g[f"{tag}_shadow_points"], LIGHT).cpu().numpy()
            assert same(occ, g[f"{tag}_shadow_occ"])
    h, t, u, v = (x.cpu().numpy() for x in kdgb_lib.trace_brute(tris, o, d))
    assert same(h, g["brute_hit"]) and same(t, g["brute_t"]) and same(u, g["brute_u"]) and same(v, g["brute_v"])
