"""Batched build + trace (kdgb_build_batch / kdgb_trace_batch): many meshes
of uneven size built as one forest; every mesh must trace exactly like its
own standalone tree does in the oracle."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
TUNED = dict(SAH_C1, mode=1, upper_levels=8, sah_bins=32)


def make_batch(n_meshes, lo, hi, rays_per_mesh, seed=40):
    sizes = np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * scenes.uniform(seed, n_meshes, 0)).astype(np.int64)
    meshes = [scenes.clustered(int(s), seed=seed + 1 + m) for m, s in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum([m.shape[0] for m in meshes])]).astype(np.int32)
    rays = [scenes.random_rays(rays_per_mesh, seed + 100 + m, t.reshape(-1, 3).min(0), t.reshape(-1, 3).max(0))
            for m, t in enumerate(meshes)]
    o = np.concatenate([r[0] for r in rays])
    d = np.concatenate([r[1] for r in rays])
    return meshes, off, o, d


@pytest.mark.parametrize("kw", [dict(), SAH_C1, TUNED], ids=["bitmap", "sah", "tuned"])
@pytest.mark.parametrize("tracer", [0, 1])
def test_batch_matches_per_mesh_oracle(kdgb_lib, cuda, oracle, kw, tracer):
    meshes, off, o, d = make_batch(10, 200, 20000, 1024)
    tris = np.concatenate(meshes)
    with kdgb_lib.KDTree.build_batch(tris, off, **kw) as tree:
        h, t, _, _ = (x.cpu().numpy() for x in tree.trace_batch(o, d, rays_per_mesh=1024, tracer=tracer,
                                                                 stack_depth=8))
    for m, mt in enumerate(meshes):
        sl = slice(1024 * m, 1024 * (m + 1))
        ref = oracle.build(mt, **kw)
        hr, tr, _, _ = oracle.trace(ref, mt, o[sl], d[sl], tracer=tracer, stack_depth=8)
        assert np.array_equal(h[sl], hr), m
        hm = hr >= 0
        assert np.array_equal(t[sl][hm].view(np.uint32), tr[hm].view(np.uint32))
    assert (h >= 0).mean() > 0.2


def test_batch_with_ray_mesh_array(kdgb_lib, cuda, oracle):
    meshes, off, o, d = make_batch(6, 100, 5000, 512, seed=60)
    tris = np.concatenate(meshes)
    owner = np.repeat(np.arange(6), 512).astype(np.int32)
    perm = (scenes.uniform(61, owner.shape[0], 0).argsort()).astype(np.int64)
    with kdgb_lib.KDTree.build_batch(tris, off) as tree:
        h_seq = tree.trace_batch(o, d, rays_per_mesh=512)[0].cpu().numpy()
        h_perm = tree.trace_batch(o[perm], d[perm], ray_mesh=owner[perm])[0].cpu().numpy()
    assert np.array_equal(h_perm, h_seq[perm])


def test_batch_validation(kdgb_lib, cuda):
    meshes, off, o, d = make_batch(3, 100, 500, 64, seed=70)
    tris = np.concatenate(meshes)
    with pytest.raises(kdgb_lib.KdgbError):
        kdgb_lib.KDTree.build_batch(tris, np.array([1, 5, 9]))  # offsets must start at 0
    with pytest.raises(kdgb_lib.KdgbError):
        kdgb_lib.KDTree.build_batch(tris, np.array([0, 50, 10, off[-1]]))  # decreasing
    with kdgb_lib.KDTree.build_batch(tris, off) as tree:
        with pytest.raises(kdgb_lib.KdgbError):
            tree.trace(o, d)  # a batch is traced with trace_batch
        with pytest.raises(kdgb_lib.KdgbError):
            tree.trace_batch(o, d, rays_per_mesh=1)  # more rays than meshes * rays_per_mesh


def test_single_mesh_batch_equals_build(kdgb_lib, cuda, oracle):
    tris = scenes.clustered(5000, seed=80)
    ref = oracle.build(tris)
    with kdgb_lib.KDTree.build_batch(tris, np.array([0, tris.shape[0]])) as tree:
        host = tree.to_host()
    assert np.array_equal(host.split.view(np.uint32), ref.split.view(np.uint32))
    assert np.array_equal(host.children, ref.children) and np.array_equal(host.prim_indices, ref.prim_indices)


@pytest.mark.parametrize("tracer", [0, 1])
def test_queue_schedule_equals_grid(kdgb_lib, cuda, tracer):
    """The persistent queue-scheduled trace (largest meshes' rays first) gives
    exactly the grid launch's results: with rays_per_mesh (mesh order), with
    a per-ray mesh array (ray order), and for one mesh traced as an image
    (4x8 packets); two launches in a row check that the queue resets."""
    meshes, off, o, d = make_batch(12, 200, 30000, 1000, seed=90)
    tris = np.concatenate(meshes)
    g = dict(tracer=tracer, stack_depth=8)
    q = dict(g, schedule=kdgb_lib._lib.SCHEDULE_QUEUE)
    with kdgb_lib.KDTree.build_batch(tris, off, **SAH_C1) as tree:
        ref = [x.cpu().numpy() for x in tree.trace_batch(o, d, rays_per_mesh=1000, **g)]
        for _ in range(2):
            got = [x.cpu().numpy() for x in tree.trace_batch(o, d, rays_per_mesh=1000, **q)]
            for a, b in zip(got, ref):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        owner = np.repeat(np.arange(12), 1000).astype(np.int32)
        got = [x.cpu().numpy() for x in tree.trace_batch(o, d, ray_mesh=owner, **q)]
        for a, b in zip(got, ref):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    one = scenes.clustered(20000, seed=91)
    o2, d2 = scenes.camera_rays(64, 48)
    with kdgb_lib.KDTree.build(one, **SAH_C1) as tree:
        ref = [x.cpu().numpy() for x in tree.trace(o2, d2, tile_width=64, **g)]
        got = [x.cpu().numpy() for x in tree.trace(o2, d2, tile_width=64, **q)]
        for a, b in zip(got, ref):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_queue_schedule_in_graph(kdgb_lib, cuda):
    """A forest rebuild + queue-scheduled trace recorded as one graph and
    launched repeatedly equals the grid-scheduled graph."""
    import torch
    meshes, off, o, d = make_batch(16, 500, 20000, 512, seed=95)
    tris = np.concatenate(meshes)
    td = torch.from_numpy(tris).cuda()
    outs = []
    for schedule in (0, 1):
        tp = kdgb_lib.trace_params(tracer=1, stack_depth=8, schedule=schedule)
        with kdgb_lib.KDTree.build_batch(td, off, **TUNED) as tree:
            g = kdgb_lib.Graph(tree, td, mesh_offsets=off, headroom=1.2, o=o, d=d, rays_per_mesh=512, trace=tp, **TUNED)
            for _ in range(3):
                g.launch()
            assert g.status() == 0
            outs.append([x.cpu().numpy() for x in g.out])
            g.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
