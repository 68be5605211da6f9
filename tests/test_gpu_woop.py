"""Woop intersection (IRayTracer::SetIntersectionAlgorithm(WOOP)): the
per-triangle transform rows of GeometryList.cu:81-102 and the test of
IRayTracer.h:78-109, bit for bit the CPU restatement's hits, for every
tracer, the fused shadow rays, the shaded loop and graph rebuilds."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)


def same(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("tracer", [0, 1, 2])
def test_woop_matches_oracle(kdgb_lib, cuda, oracle, tracer):
    tris = scenes.clustered(8000, seed=51)
    o, d = scenes.camera_rays(96, 64)
    ref = oracle.build(tris, **SAH_C1)
    hr, tr, ur, vr = oracle.trace(ref if tracer != 2 else None, tris, o, d, tracer=tracer, intersection=1)
    with kdgb_lib.KDTree.build(tris, **SAH_C1) as tree:
        h, t, u, v = (x.cpu().numpy() for x in tree.trace(o, d, tracer=tracer, intersection=1))
        hm = tree.trace(o, d, tracer=tracer)[0].cpu().numpy()
    assert np.array_equal(h, hr)
    m = hr >= 0
    assert same(t[m], tr[m]) and same(u[m], ur[m]) and same(v[m], vr[m])
    assert m.mean() > 0.3
    # Woop and Moeller-Trumbore agree on nearly every hit
    assert (h == hm).mean() > 0.99


def test_woop_brute_without_tree(kdgb_lib, cuda, oracle):
    import ctypes as C
    import torch
    tris = scenes.clustered(1500, seed=52)
    o, d = scenes.camera_rays(48, 32)
    hr, tr, _, _ = oracle.trace(None, tris, o, d, tracer=2, intersection=1)
    td, od, dd = (torch.from_numpy(x).cuda() for x in (tris, o, d))
    n = o.shape[0]
    out = [torch.empty(n, dtype=torch.int32, device="cuda")] + [torch.empty(n, device="cuda") for _ in range(3)]
    p = kdgb_lib.trace_params(intersection=1)
    ptr = lambda x: C.c_void_p(x.data_ptr())
    kdgb_lib.check(kdgb_lib.lib().kdgb_trace_brute_ex(ptr(td), tris.shape[0], C.byref(p), ptr(od), ptr(dd), n,
                                                      *[ptr(x) for x in out], None), "brute_ex")
    assert np.array_equal(out[0].cpu().numpy(), hr)
    m = hr >= 0
    assert same(out[1].cpu().numpy()[m], tr[m])


def test_woop_fused_shadow_and_shading(kdgb_lib, cuda, oracle):
    tris, n0, n1, n2, c0 = scenes.shaded_box(24, 12, seed=5)
    o, d = scenes.camera_rays(64, 32)
    ref = oracle.build(tris)
    light = (0.5, 3.0, 0.5)
    with kdgb_lib.KDTree.build(tris) as tree:
        h, t, _, _, occ = (x.cpu().numpy() for x in tree.trace_primary_shadow(o, d, light, tracer=1, intersection=1))
        px = tree.trace_shaded(o, d, n0, n1, n2, c0, tracer=0, intersection=1).cpu().numpy()
    hr, tr, _, _ = oracle.trace(ref, tris, o, d, tracer=1, intersection=1)
    assert np.array_equal(h, hr)
    pts = scenes.hit_points(o, d, tr, hr)[hr >= 0]
    occ_r = oracle.trace_shadow(ref, tris, pts, light, intersection=1)
    assert np.array_equal(occ[hr >= 0], occ_r)
    want = oracle.trace_shaded(ref, tris, o, d, n0, n1, n2, c0, tracer=0, intersection=1)
    assert np.array_equal(px, want)


def test_woop_rows_follow_graph_rebuilds(kdgb_lib, cuda, oracle):
    import torch
    verts0 = scenes.heightfield_vertices(32, 16, seed=6)
    idx = scenes.grid_indices(32, 16).astype(np.int64)

    def frame(k):
        v = verts0.copy()
        v[:, 2] += 0.05 * np.sin(0.9 * k + 4.0 * v[:, 1])
        return np.ascontiguousarray(v[idx].reshape(-1, 9), dtype=np.float32)

    o, d = scenes.camera_rays(32, 32)
    tp = kdgb_lib.trace_params(tracer=1, intersection=1)
    with kdgb_lib.KDTree.build(frame(0)) as tree:
        td = torch.from_numpy(frame(0)).cuda()
        tree.trace(o, d, tp)  # fills the Woop cache for frame 0
        g = kdgb_lib.Graph(tree, td, headroom=2.0, o=o, d=d, trace=tp)
        for k in (1, 2):
            td.copy_(torch.from_numpy(frame(k)))
            g.launch()
            assert g.status() == 0
            ref = oracle.build(frame(k))
            hr, _, _, _ = oracle.trace(ref, frame(k), o, d, tracer=1, intersection=1)
            assert np.array_equal(g.out[0].cpu().numpy(), hr)
            # a plain trace after the graph launch recomputes the rows too
            assert np.array_equal(tree.trace(o, d, tp)[0].cpu().numpy(), hr)
        g.close()
