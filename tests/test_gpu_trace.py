"""GPU traversal parity: kd-restart, short-stack, brute force and shadow rays
of libkdgb.so against the oracle on the same tree and the same rays.  Hit ids
are compared bit for bit; t, u, v too (the arithmetic is the same, so the
1e-6 relative tolerance of the contract is not needed, but it is asserted as
the documented bound)."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-6  # contract tolerance on t, u, v


def np_(x):
    return x.cpu().numpy()


def assert_hits_equal(got, ref, exact=True):
    h, t, u, v = (np_(x) for x in got)
    hr, tr, ur, vr = ref
    assert np.array_equal(h, hr), f"{(h != hr).sum()} hit ids differ"
    hitm = hr >= 0
    for a, b in ((t, tr), (u, ur), (v, vr)):
        assert np.allclose(a[hitm], b[hitm], rtol=RTOL, atol=0)
        if exact:
            assert np.array_equal(a[hitm].view(np.uint32), b[hitm].view(np.uint32))
    assert np.isinf(t[~hitm]).all()


@pytest.fixture(scope="module")
def c1(oracle):
    tris = scenes.heightfield(64, 32, seed=1)[0]
    o, d = scenes.camera_rays(256, 256)
    return tris, oracle.build(tris), o, d


@pytest.fixture(scope="module")
def clustered(oracle):
    tris = scenes.clustered(30000, seed=6)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    o, d = scenes.random_rays(20000, 7, lo, hi)
    o2, d2 = scenes.camera_rays(128, 96)
    return tris, oracle.build(tris), np.concatenate([o, o2]), np.concatenate([d, d2])


@pytest.mark.parametrize("tracer", [0, 1])
@pytest.mark.parametrize("skip", [0, 1])
@pytest.mark.parametrize("tie", [0, 1])
def test_kd_tracers_on_uploaded_tree(kdgb_lib, cuda, oracle, clustered, tracer, skip, tie):
    tris, tree, o, d = clustered
    ref = oracle.trace(tree, tris, o, d, tracer=tracer, leaf_skipping=skip, tie=tie)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        got = gt.trace(o, d, tracer=tracer, leaf_skipping=skip, tie=tie)
        assert_hits_equal(got, ref)


@pytest.mark.parametrize("depth", [1, 2, 3, 4, 8])
def test_shortstack_depths(kdgb_lib, cuda, oracle, clustered, depth):
    tris, tree, o, d = clustered
    ref = oracle.trace(tree, tris, o, d, tracer=1, stack_depth=depth)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        assert_hits_equal(gt.trace(o, d, tracer=1, stack_depth=depth), ref)


@pytest.mark.parametrize("tie", [0, 1])
def test_brute_force(kdgb_lib, cuda, oracle, c1, tie):
    tris, _, o, d = c1
    ref = oracle.trace(None, tris, o, d, tracer=2, tie=tie)
    assert_hits_equal(kdgb_lib.trace_brute(tris, o, d, tie=tie), ref)


@pytest.mark.parametrize("lower", [0, 1])
@pytest.mark.parametrize("tracer", [0, 1, 2])
def test_gpu_built_tree_traces_like_oracle(kdgb_lib, cuda, oracle, c1, lower, tracer):
    tris, _, o, d = c1
    kw = dict(lower=lower)
    if lower == 1:
        kw.update(traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)  # C1 SAH settings
    ref_tree = oracle.build(tris, **kw)
    ref = oracle.trace(ref_tree, tris, o, d, tracer=tracer)
    with kdgb_lib.KDTree.build(tris, **kw) as gt:
        assert_hits_equal(gt.trace(o, d, tracer=tracer), ref)


def test_tile_remap_is_transparent(kdgb_lib, cuda, oracle, c1):
    tris, tree, o, d = c1
    ref = oracle.trace(tree, tris, o, d, tracer=1)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        assert_hits_equal(gt.trace(o, d, tracer=1, tile_width=256), ref)
        assert_hits_equal(gt.trace(o, d, tracer=0, tile_width=256, block_size=64),
                          oracle.trace(tree, tris, o, d, tracer=0))


def test_shadow_rays(kdgb_lib, cuda, oracle, clustered):
    tris, tree, o, d = clustered
    hb, tb, _, _ = oracle.trace(tree, tris, o, d, tracer=0)
    pts = scenes.hit_points(o, d, tb, hb)[hb >= 0]
    light = (0.5, 3.0, 0.5)
    ref = oracle.trace_shadow(tree, tris, pts, light)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        occ = np_(gt.trace_shadow(pts, light))
    assert np.array_equal(occ, ref)
    assert ref.sum() > 0


@pytest.mark.parametrize("tracer", [0, 1])
@pytest.mark.parametrize("block_size", [0, 64, 1024])
def test_fused_primary_shadow(kdgb_lib, cuda, oracle, clustered, tracer, block_size):
    """Shadow rays are packed onto a block's first threads; 1024-thread
    blocks need more than 48 KB of shared memory."""
    tris, tree, o, d = clustered
    light = (0.5, 3.0, 0.5)
    ref = oracle.trace(tree, tris, o, d, tracer=tracer, stack_depth=8)
    pts = scenes.hit_points(o, d, ref[1], ref[0])
    occ_ref = oracle.trace_shadow(tree, tris, pts, light)
    occ_ref[ref[0] < 0] = 0
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        h, t, u, v, occ = gt.trace_primary_shadow(o, d, light, tracer=tracer, stack_depth=8, block_size=block_size)
        assert_hits_equal((h, t, u, v), ref)
        assert np.array_equal(np_(occ), occ_ref)


@pytest.mark.parametrize("depth", [1, 2, 3])
def test_fused_shadow_small_memo(kdgb_lib, cuda, oracle, clustered, depth):
    """The fused launch's shadow rays remember their descents in the primary
    ray's stack region: 1 or 2 entries at these depths, so the ring drops
    entries and restarts from the root on most rays (with 8 entries it hardly
    ever does on this scene)."""
    tris, tree, o, d = clustered
    light = (0.5, 3.0, 0.5)
    ref = oracle.trace(tree, tris, o, d, tracer=1, stack_depth=depth)
    pts = scenes.hit_points(o, d, ref[1], ref[0])
    occ_ref = oracle.trace_shadow(tree, tris, pts, light)
    occ_ref[ref[0] < 0] = 0
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        h, t, u, v, occ = gt.trace_primary_shadow(o, d, light, tracer=1, stack_depth=depth)
        assert_hits_equal((h, t, u, v), ref)
        assert np.array_equal(np_(occ), occ_ref)
    assert occ_ref.sum() > 100


def test_step_counts(kdgb_lib, cuda, oracle, clustered):
    """kdgb_trace_count_steps: the fused launch compiled with counters writes
    the outputs of the timed launch, counts the same twice, and its counts
    agree with what the outputs imply."""
    tris, tree, o, d = clustered
    light = (0.5, 3.0, 0.5)
    kw = dict(tracer=1, stack_depth=8)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        ref = [np_(x) for x in gt.trace_primary_shadow(o, d, light, **kw)]
        outs, steps = gt.count_steps(o, d, light, **kw)
        _, again = gt.count_steps(o, d, light, **kw)
        with pytest.raises(kdgb_lib.KdgbError):
            gt.count_steps(o, d, light, tracer=0)
    for a, b in zip((np_(x) for x in outs), ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert steps == again
    p, s = steps["primary"], steps["shadow"]
    n, hits, occluded = o.shape[0], int((ref[0] >= 0).sum()), int(ref[4].sum())
    assert p["leaf"] >= n and p["node"] >= p["leaf"]
    assert p["box"] == p["leaf"]  # leaf skipping: one box per leaf reached
    assert p["tri"] >= hits
    assert s["box"] == 0 and s["leaf"] >= hits and s["node"] >= s["leaf"]
    assert s["tri"] >= occluded > 0


def test_edge_case_rays(kdgb_lib, cuda, oracle):
    tris = scenes.heightfield(16, 16, seed=2)[0]
    tree = oracle.build(tris)
    o = np.array([[0.3, 0.3, 2.0], [0.7, 0.2, 2.0], [0.3, 0.3, 2.0], [0.5, 0.5, 0.5], [5, 5, 5],
                  [0.25, 0.25, 2.0]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, -1], [1, 0, 0], [0, 0, 1], [1, 1, 1], [1e-30, -1e-30, -1]], np.float32)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        for tracer in (0, 1):
            assert_hits_equal(gt.trace(o, d, tracer=tracer), oracle.trace(tree, tris, o, d, tracer=tracer))
    assert_hits_equal(kdgb_lib.trace_brute(tris, o, d), oracle.trace(None, tris, o, d, tracer=2))


def test_empty_scene_and_zero_rays(kdgb_lib, cuda, oracle):
    empty = np.zeros((0, 9), np.float32)
    o, d = scenes.camera_rays(16, 16)
    with kdgb_lib.KDTree.build(empty) as gt:
        h, t, _, _ = gt.trace(o, d)
        assert (np_(h) == -1).all() and np.isinf(np_(t)).all()
        out = gt.trace(o[:0], d[:0])
        assert out[0].numel() == 0


def test_invalid_trace_params(kdgb_lib, cuda, c1):
    tris, tree, o, d = c1
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        for bad in (dict(tracer=9), dict(stack_depth=0), dict(stack_depth=9), dict(block_size=33),
                    dict(tile_width=250)):
            with pytest.raises(kdgb_lib.KdgbError) as e:
                gt.trace(o, d, **bad)
            assert e.value.status == 1


def test_upload_rejects_malformed_tree(kdgb_lib, cuda, oracle, c1):
    tris, tree, _, _ = c1
    import copy
    bad = copy.deepcopy(tree)
    interior = np.nonzero(bad.info != 0)[0][0]
    bad.children[interior, 0] = bad.n_nodes + 5
    with pytest.raises(kdgb_lib.KdgbError) as e:
        kdgb_lib.KDTree.upload(bad, tris)
    assert e.value.status == 1


def test_fp64_error_reported(kdgb_lib, cuda, oracle, c1):
    tris, tree, o, d = c1
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        h, t, u, v = (np_(x) for x in gt.trace(o, d, tracer=0))
    hf, tf, uf, vf = oracle.trace_brute_f64(tris, o, d)
    agree = (h == hf) & (h >= 0)
    assert agree.mean() > 0.3
    rel = np.abs(t[agree] - tf[agree]) / np.abs(tf[agree])
    assert rel.max() < 1e-5
