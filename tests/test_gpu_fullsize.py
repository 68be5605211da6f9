"""Parity at the sizes the measured numbers are quoted on.

* frame: the 1,000,000-triangle clustered scene rebuilt by one graph launch
  exactly as bench.py runs it (both the frame's tuned build and the
  reference creators), every tree array against the oracle, and the fused
  short-stack primary + shadow trace over the full 1920x1080 frame (4x8
  pixel packets, depth 8) and kd-restart over the same frame, bit for bit;
* photons: the 262,144-triangle scene with a 1M-photon sample of the 16M
  photon stream, both kd tracers;
* batched: 64 meshes drawn from the log-uniform 1k..200k mix, one forest
  graph (build + batched trace) against each mesh's own oracle tree.

The oracle runs these sizes in seconds on the host cores (OpenMP)."""
import numpy as np
import pytest

from kdgb import configs, scenes

pytestmark = pytest.mark.gpu

FIELDS = ("info", "split", "children", "prim_index", "bitmap", "parent", "area", "aabb_min", "aabb_max",
          "prim_indices", "leaf_ids")


def assert_same_tree(gpu, ref):
    for f in FIELDS:
        a, b = getattr(gpu, f), getattr(ref, f)
        assert a.shape == b.shape, (f, a.shape, b.shape)
        if a.dtype.kind == "f":
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f
        else:
            assert np.array_equal(a, b), f


def np_(x):
    return x.cpu().numpy()


@pytest.fixture(scope="module")
def frame():
    return configs.frame_scene()


@pytest.mark.parametrize("build", ["tuned", "reference"])
def test_frame_build_and_trace_match_oracle(kdgb_lib, cuda, oracle, frame, build):
    import torch
    tris, o, d = frame
    kw = configs.TUNED if build == "tuned" else configs.SAH
    ref_tree = oracle.build(tris, **kw)
    td = torch.from_numpy(tris).cuda()
    bp = kdgb_lib.build_params(**kw)
    tp = kdgb_lib.trace_params(tracer=kdgb_lib.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH,
                               tile_width=configs.WIDTH)
    with kdgb_lib.KDTree.build(td, bp) as tree:
        assert_same_tree(tree.to_host(), ref_tree)
        g = kdgb_lib.Graph(tree, td, params=bp, headroom=1.1)
        for _ in range(2):  # the graph replay rebuilds from scratch each launch
            g.launch()
        assert g.status() == 0
        assert_same_tree(tree.to_host(), ref_tree)
        h, t, u, v, occ = (np_(x) for x in tree.trace_primary_shadow(o, d, configs.LIGHT, tp))
        # kd-restart over the same frame: its descents run deep enough here
        # to overflow the 8-entry ring of remembered descents.
        restart = [np_(x) for x in tree.trace(o, d, tracer=kdgb_lib.TRACER_RESTART, tile_width=configs.WIDTH)]
        g.close()
    hr, tr, ur, vr = oracle.trace(ref_tree, tris, o, d, tracer=1, stack_depth=configs.STACK_DEPTH)
    assert np.array_equal(h, hr), f"{(h != hr).sum()} of {h.size} hit ids differ"
    m = hr >= 0
    assert m.mean() > 0.3
    for a, b in ((t, tr), (u, ur), (v, vr)):
        assert np.array_equal(a[m].view(np.uint32), b[m].view(np.uint32))
    assert np.isinf(t[~m]).all()
    pts = scenes.hit_points(o, d, tr, hr)
    occ_ref = oracle.trace_shadow(ref_tree, tris, pts[m], configs.LIGHT)
    assert np.array_equal(occ[m], occ_ref), f"{(occ[m] != occ_ref).sum()} shadow rays differ"
    assert (occ[~m] == 0).all()
    assert 0 < occ_ref.sum() < occ_ref.size
    hk, tk, uk, vk = oracle.trace(ref_tree, tris, o, d, tracer=0)
    assert np.array_equal(restart[0], hk), f"{(restart[0] != hk).sum()} kd-restart hit ids differ"
    mk = hk >= 0
    for a, b in zip(restart[1:], (tk, uk, vk)):
        assert np.array_equal(a[mk].view(np.uint32), b[mk].view(np.uint32))


@pytest.mark.parametrize("tracer", [0, 1])
def test_photons_full_scene_match_oracle(kdgb_lib, cuda, oracle, tracer):
    tris = scenes.clustered(configs.PHOTON_TRIS, seed=configs.FRAME_SEED)
    ref_tree = oracle.build(tris, **configs.SAH)
    n = 1 << 20
    kw = dict(light=configs.LIGHT, seed=configs.PHOTON_SEED, bounces=configs.PHOTON_BOUNCES,
              survival=configs.PHOTON_SURVIVAL)
    ref_h, ref_t = oracle.trace_photons(ref_tree, tris, n, tracer=tracer, stack_depth=configs.STACK_DEPTH, **kw)
    with kdgb_lib.KDTree.build(tris, **configs.SAH) as gt:
        assert_same_tree(gt.to_host(), ref_tree)
        h, t = (np_(x) for x in gt.trace_photons(n, photons=kdgb_lib.photon_params(**kw), tracer=tracer,
                                                  stack_depth=configs.STACK_DEPTH))
    assert np.array_equal(h, ref_h), f"{(h != ref_h).sum()} segment ids differ"
    m = ref_h >= 0
    assert np.array_equal(t[m].view(np.uint32), ref_t[m].view(np.uint32))
    # Photons leave the light above the scene in all directions: about half
    # head up and miss; every bounce level still has hits.
    assert all((ref_h[:, k] >= 0).sum() > 100 for k in range(configs.PHOTON_BOUNCES + 1))


def test_batched_64_meshes_match_oracle(kdgb_lib, cuda, oracle):
    import torch
    R = 4096
    meshes, off, o, d = configs.batch_scene(n_meshes=64, rays_per_mesh=R)
    tris = np.concatenate(meshes)
    assert tris.shape[0] > 1_000_000
    kw = configs.TUNED
    bp = kdgb_lib.build_params(**kw)
    tp = kdgb_lib.trace_params(tracer=kdgb_lib.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH)
    td = torch.from_numpy(tris).cuda()
    refs = [oracle.build(mt, **kw) for mt in meshes]
    with kdgb_lib.KDTree.build_batch(td, off, bp) as forest:
        st = forest.stats()
        assert st.n_nodes == sum(r.n_nodes for r in refs)
        assert st.n_refs == sum(r.prim_indices.shape[0] for r in refs)
        g = kdgb_lib.Graph(forest, td, mesh_offsets=off, params=bp, headroom=1.1, o=o, d=d, rays_per_mesh=R,
                           trace=tp)
        g.launch()
        g.launch()
        assert g.status() == 0
        h, t, u, v = (np_(x) for x in g.out)
        g.close()
    for m, mt in enumerate(meshes):
        sl = slice(R * m, R * (m + 1))
        hr, tr, ur, vr = oracle.trace(refs[m], mt, o[sl], d[sl], tracer=1, stack_depth=configs.STACK_DEPTH)
        assert np.array_equal(h[sl], hr), m
        hm = hr >= 0
        for a, b in ((t, tr), (u, ur), (v, vr)):
            assert np.array_equal(a[sl][hm].view(np.uint32), b[hm].view(np.uint32)), m
    assert (h >= 0).mean() > 0.2
