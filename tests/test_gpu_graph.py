"""Graph rebuilds (kdgb_graph_*): one CUDA graph whose level loops are
conditional WHILE nodes must build exactly the tree the host-driven build
makes, rebuild changed geometry refilled in place, and stop cleanly when the
geometry outgrows its fixed buffers."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

FIELDS = ("info", "split", "children", "prim_index", "bitmap", "parent", "area", "aabb_min", "aabb_max",
          "prim_indices", "leaf_ids")
SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
TUNED = dict(SAH_C1, mode=1, upper_levels=8, sah_bins=16)
CONFIGS = {"bitmap": dict(), "sah": SAH_C1, "tuned": TUNED, "no_ess": dict(split_empty_space=0),
           "balanced_divide": dict(lower=2, split_method=1),
           # binned SAH from level 1: nodes of ~10k references binned in chunks by several blocks
           "tuned_sah_from_level1": dict(SAH_C1, mode=1, upper_levels=1, sah_bins=32)}


def assert_same_tree(a, b):
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert x.shape == y.shape, f
        if x.dtype.kind == "f":
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), f
        else:
            assert np.array_equal(x, y), f


def host_tree(kdgb_lib, tris, kw):
    with kdgb_lib.KDTree.build(tris, **kw) as t:
        return t.to_host(), t.stats()


@pytest.mark.parametrize("cfg", list(CONFIGS))
def test_graph_rebuild_matches_host_build(kdgb_lib, cuda, oracle, cfg):
    import torch
    kw = CONFIGS[cfg]
    tris = scenes.clustered(20000, seed=11)
    o, d = scenes.camera_rays(64, 48)
    ref, ref_stats = host_tree(kdgb_lib, tris, kw)
    tp = kdgb_lib.trace_params(tracer=1, stack_depth=4)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        td = torch.from_numpy(tris).cuda()
        g = kdgb_lib.Graph(tree, td, headroom=1.25, o=o, d=d, trace=tp, **kw)
        for _ in range(3):  # replays rebuild from scratch every launch
            g.launch()
            assert g.status() == 0
        assert_same_tree(tree.to_host(), ref)
        st = tree.stats()
        assert (st.n_nodes, st.n_refs, st.upper_levels, st.lower_levels) == \
            (ref_stats.n_nodes, ref_stats.n_refs, ref_stats.upper_levels, ref_stats.lower_levels)
        h = g.out[0].cpu().numpy()
        t = g.out[1].cpu().numpy()
        hr, tr, _, _ = (x.cpu().numpy() for x in tree.trace(o, d, tp))
        assert np.array_equal(h, hr) and np.array_equal(t.view(np.uint32), tr.view(np.uint32))
        # and the oracle agrees on the trace
        otree = oracle.build(tris, **kw)
        ho, _, _, _ = oracle.trace(otree, tris, o, d, tracer=1, stack_depth=4)
        assert np.array_equal(h, ho)
        g.close()


def test_graph_rebuilds_refilled_geometry(kdgb_lib, cuda, oracle):
    """The oscillating height field: one graph, geometry moved in place
    between launches, every launch equal to a fresh build."""
    import torch
    verts0 = scenes.heightfield_vertices(48, 24, seed=3)
    idx = scenes.grid_indices(48, 24).astype(np.int64)

    def frame(k):
        v = verts0.copy()
        v[:, 2] += 0.05 * np.sin(0.7 * k + 3.0 * v[:, 0])
        return np.ascontiguousarray(v[idx].reshape(-1, 9), dtype=np.float32)

    o, d = scenes.camera_rays(32, 32)
    kw = SAH_C1
    with kdgb_lib.KDTree.build(frame(0), **kw) as tree:
        td = torch.from_numpy(frame(0)).cuda()
        g = kdgb_lib.Graph(tree, td, headroom=2.0, o=o, d=d, **kw)
        for k in range(1, 4):
            td.copy_(torch.from_numpy(frame(k)))
            g.launch()
            assert g.status() == 0
            ref, _ = host_tree(kdgb_lib, frame(k), kw)
            assert_same_tree(tree.to_host(), ref)
            otree = oracle.build(frame(k), **kw)
            ho, to, _, _ = oracle.trace(otree, frame(k), o, d)
            assert np.array_equal(g.out[0].cpu().numpy(), ho)
        g.close()


def test_graph_batch_matches_batch_build(kdgb_lib, cuda):
    import torch
    sizes = [300, 5000, 40, 12000, 800]
    meshes = [scenes.clustered(s, seed=90 + i) for i, s in enumerate(sizes)]
    tris = np.concatenate(meshes)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    rays = [scenes.random_rays(256, 200 + m, t.reshape(-1, 3).min(0), t.reshape(-1, 3).max(0))
            for m, t in enumerate(meshes)]
    o = np.concatenate([r[0] for r in rays])
    d = np.concatenate([r[1] for r in rays])
    for kw in (dict(), SAH_C1):
        with kdgb_lib.KDTree.build_batch(tris, off, **kw) as ref_tree:
            ref = ref_tree.to_host()
            hr = ref_tree.trace_batch(o, d, rays_per_mesh=256)[0].cpu().numpy()
        with kdgb_lib.KDTree.build_batch(tris, off, **kw) as tree:
            g = kdgb_lib.Graph(tree, torch.from_numpy(tris).cuda(), mesh_offsets=off, o=o, d=d, rays_per_mesh=256,
                               **kw)
            g.launch()
            assert g.status() == 0
            assert_same_tree(tree.to_host(), ref)
            assert np.array_equal(g.out[0].cpu().numpy(), hr)
            g.close()


def test_graph_capacity_stop(kdgb_lib, cuda):
    """Geometry that outgrows the fixed buffers: the launch stops with
    KDGB_ERR_CAPACITY, traces report misses, a host rebuild recovers."""
    import torch
    T = 131072
    flat = scenes.heightfield(256, 256, seed=1, amplitude=0.0)[0]  # 131,072 triangles in a plane
    assert flat.shape[0] == T
    busy = scenes.clustered(T, seed=12)
    o, d = scenes.camera_rays(32, 32)
    with kdgb_lib.KDTree.build(flat) as tree:
        td = torch.from_numpy(flat).cuda()
        g = kdgb_lib.Graph(tree, td, headroom=1.0, o=o, d=d)
        g.launch()
        assert g.status() == 0
        td.copy_(torch.from_numpy(busy))
        g.launch()
        assert g.status() == kdgb_lib.ERR_CAPACITY
        assert (g.out[0].cpu().numpy() == -1).all()
        # The queue-scheduled trace of the failed tree reports misses too, and
        # leaves its queue ready for the next launch.
        for _ in range(2):
            h, t, _, _ = tree.trace(o, d, schedule=kdgb_lib.SCHEDULE_QUEUE)
            assert (h.cpu().numpy() == -1).all() and torch.isinf(t).all()
        g.close()
        tree.rebuild(busy)
        ref, _ = host_tree(kdgb_lib, busy, {})
        assert_same_tree(tree.to_host(), ref)


def test_graph_invalidated_by_reallocation(kdgb_lib, cuda):
    import torch
    small = scenes.clustered(2000, seed=13)
    with kdgb_lib.KDTree.build(small) as tree:
        g = kdgb_lib.Graph(tree, torch.from_numpy(small).cuda())
        g.launch()
        assert g.status() == 0
        tree.rebuild(scenes.clustered(200000, seed=14))  # grows every buffer
        with pytest.raises(kdgb_lib.KdgbError) as e:
            g.launch()
        assert e.value.status == kdgb_lib.ERR_INVALID_ARGUMENT
        g.close()


def test_graph_requires_a_build(kdgb_lib, cuda):
    import torch
    tris = scenes.clustered(1000, seed=15)
    with kdgb_lib.KDTree.build(tris) as tree:
        with pytest.raises(kdgb_lib.KdgbError):
            kdgb_lib.Graph(tree, torch.from_numpy(tris).cuda(), headroom=0.5)
