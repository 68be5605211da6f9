"""GPU build parity: every build of libkdgb.so (reference and tuned modes,
BITMAP / SAH / BALANCED lower creators, BOX / DIVIDE split methods) must
produce the oracle's tree bit for bit (node arrays, leaf lists, reference
order)."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

FIELDS = ("info", "split", "children", "prim_index", "bitmap", "parent", "area", "aabb_min", "aabb_max",
          "prim_indices", "leaf_ids")


def tri_soup(n, seed, scale=0.05):
    c = np.stack([scenes.uniform(seed, n, k) for k in range(3)], axis=1)
    off = (np.stack([scenes.uniform(seed, n, 10 + k) for k in range(9)], axis=1) - 0.5) * scale
    return np.ascontiguousarray((np.tile(c, 3) + off).astype(np.float32))


def assert_same_tree(gpu, ref):
    assert gpu.info.shape == ref.info.shape, (gpu.info.shape, ref.info.shape)
    for f in FIELDS:
        a, b = getattr(gpu, f), getattr(ref, f)
        assert a.shape == b.shape, f
        if a.dtype.kind == "f":
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f
        else:
            assert np.array_equal(a, b), f


def scene(name):
    if name == "c1":
        return scenes.heightfield(64, 32, seed=1)[0]
    if name == "clustered3k":
        return scenes.clustered(3000, seed=4)
    if name == "clustered60k":
        return scenes.clustered(60000, seed=5)
    if name == "soup":
        return tri_soup(5000, 7)
    if name == "degenerate":
        t = tri_soup(600, 8)
        t[::7, 3:6] = t[::7, 0:3]          # zero-area triangles
        t[::11, 6:9] = t[::11, 3:6]
        return t
    raise KeyError(name)


@pytest.mark.parametrize("name", ["c1", "clustered3k", "clustered60k", "soup", "degenerate"])
@pytest.mark.parametrize("lower", [0, 1, 2])
def test_build_matches_oracle(kdgb_lib, cuda, oracle, name, lower):
    tris = scene(name)
    ref = oracle.build(tris, lower=lower)
    with kdgb_lib.KDTree.build(tris, lower=lower) as tree:
        assert_same_tree(tree.to_host(), ref)
        st = tree.stats()
        assert st.upper_levels == ref.upper_levels and st.n_nodes == ref.n_nodes


@pytest.mark.parametrize("opts", [
    dict(split_empty_space=0),
    dict(split_empty_space=0, propagate_aabbs=0),
    dict(esc_zmax_as_x=0),
    dict(leaf_size=8),
    dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8),
    dict(lower=1, propagate_aabbs=0),
    dict(empty_space_threshold=0.1),
    dict(lower=2, traversal_cost=16.0),
    dict(lower=2, traversal_cost=0.0, propagate_aabbs=0),
    dict(lower=2, leaf_size=12),
])
def test_build_options_match_oracle(kdgb_lib, cuda, oracle, opts):
    tris = scenes.clustered(8000, seed=14)
    ref = oracle.build(tris, **opts)
    with kdgb_lib.KDTree.build(tris, **opts) as tree:
        assert_same_tree(tree.to_host(), ref)


@pytest.mark.parametrize("min_leaf,ci", [(0, 1.5), (4, 1.5), (15, 1.5), (16, 4.0), (20, 8.0), (31, 1.5)])
def test_sah_lower_work_lists_match_oracle(kdgb_lib, cuda, oracle, min_leaf, ci):
    """The SAH lower levels evaluate the nodes with more than min_leaf members
    from work lists, two nodes of at most 16 members per warp and larger ones
    one per warp; min_leaf moves the split between the two kinds (0: every
    node with a member, 16: no pairs at all, 31: nothing after the first
    level).  Host-driven and graph rebuilds must give the oracle's tree."""
    kw = dict(lower=1, traversal_cost=1.0, intersection_cost=ci, min_leaf=min_leaf)
    tris = scenes.clustered(12000, seed=33)
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        assert_same_tree(tree.to_host(), ref)
        params = kdgb_lib.build_params(**kw)
        with kdgb_lib.Graph(tree, tris, params=params, headroom=1.5) as g:
            g.launch()
            assert g.status() == 0
            assert_same_tree(tree.to_host(), ref)


TUNED = dict(mode=1, upper_levels=8, sah_bins=32, lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)


@pytest.mark.parametrize("name", ["c1", "clustered3k", "clustered60k", "soup", "degenerate"])
def test_tuned_build_matches_oracle(kdgb_lib, cuda, oracle, name):
    """Tuned mode (median for 8 levels, then binned SAH; empty-space cuts on
    every level) has no reference counterpart; the oracle restates it, so the
    trees must be identical."""
    tris = scene(name)
    ref = oracle.build(tris, **TUNED)
    with kdgb_lib.KDTree.build(tris, **TUNED) as tree:
        assert_same_tree(tree.to_host(), ref)


@pytest.mark.parametrize("opts", [dict(upper_levels=0), dict(upper_levels=3, sah_bins=8), dict(sah_bins=2),
                                  dict(upper_levels=40)])
def test_tuned_build_options(kdgb_lib, cuda, oracle, opts):
    kw = dict(TUNED, **opts)
    tris = scenes.clustered(20000, seed=16)
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        assert_same_tree(tree.to_host(), ref)


def test_tuned_build_large_nodes(kdgb_lib, cuda, oracle):
    """Binned SAH from level 2 of a 300k-triangle scene: nodes of about 75k
    references are binned in 2048-reference chunks by many blocks, whose
    histograms meet in global memory; the tree must still be the oracle's."""
    kw = dict(TUNED, upper_levels=2)
    tris = scenes.clustered(300000, seed=23)
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        assert_same_tree(tree.to_host(), ref)


@pytest.mark.parametrize("name", ["c1", "clustered3k", "clustered60k", "soup", "degenerate"])
@pytest.mark.parametrize("lower", [0, 2])
def test_divide_build_matches_oracle(kdgb_lib, cuda, oracle, name, lower):
    """The DIVIDE split method (triangle against the two half boxes of a
    straddled node) builds the oracle's tree bit for bit."""
    tris = scene(name)
    kw = dict(split_method=1, lower=lower)
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        assert_same_tree(tree.to_host(), ref)


def test_divide_drops_references_and_traces_like_brute_force(kdgb_lib, cuda, oracle):
    tris = tri_soup(20000, 31, scale=0.08)
    o, d = scenes.camera_rays(96, 64)
    with kdgb_lib.KDTree.build(tris) as box, kdgb_lib.KDTree.build(tris, split_method=1, lower=2) as div:
        assert div.stats().n_refs < box.stats().n_refs
        brute = [x.cpu().numpy() for x in kdgb_lib.trace_brute(tris, o, d)]
        for tracer in (0, 1):
            got = [x.cpu().numpy() for x in div.trace(o, d, tracer=tracer)]
            assert np.array_equal(got[0], brute[0]), tracer
            if tracer == 0:
                assert np.array_equal(got[1].view(np.uint32), brute[1].view(np.uint32))
            else:  # the short stack measures t from a moved origin
                assert np.allclose(got[1], brute[1], rtol=1e-5)


def test_tuned_divide_balanced_matches_oracle(kdgb_lib, cuda, oracle):
    kw = dict(TUNED, split_method=1, lower=2, traversal_cost=16.0)
    tris = scenes.clustered(30000, seed=19)
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        assert_same_tree(tree.to_host(), ref)


@pytest.mark.parametrize("T", [0, 1, 2, 31, 32, 33, 257])
@pytest.mark.parametrize("kw", [dict(), dict(lower=2, split_method=1)])
def test_small_and_empty_builds(kdgb_lib, cuda, oracle, T, kw):
    tris = tri_soup(max(T, 1), 30)[:T]
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, **kw) as tree:
        assert_same_tree(tree.to_host(), ref)


def test_rebuild_reuses_handle(kdgb_lib, cuda, oracle):
    a, b = scenes.clustered(20000, seed=1), scenes.heightfield(40, 30, seed=3)[0]
    with kdgb_lib.KDTree.build(a) as tree:
        tree.rebuild(b, lower=1)
        assert_same_tree(tree.to_host(), oracle.build(b, lower=1))
        tree.rebuild(a)
        assert_same_tree(tree.to_host(), oracle.build(a))


@pytest.mark.parametrize("lower", [1, 2])
def test_rebuild_grows_lower_decision_arrays(kdgb_lib, cuda, oracle, lower):
    """A handle first built over a small scene (small lower-phase arrays)
    rebuilt host-driven over one with many more upper leaves: the first
    lower level's decisions, which the plane kernel writes before the lower
    loop starts, must survive the arrays' growth."""
    kw = dict(configs_sah(), lower=lower)
    small, big = scenes.clustered(500, seed=41), scenes.clustered(60000, seed=42)
    with kdgb_lib.KDTree.build(small, **kw) as tree:
        tree.rebuild(big, **kw)
        assert_same_tree(tree.to_host(), oracle.build(big, **kw))
        tree.rebuild(small, **kw)
        assert_same_tree(tree.to_host(), oracle.build(small, **kw))


def configs_sah():
    from kdgb import configs
    return dict(configs.SAH)


def test_nonfinite_is_an_error(kdgb_lib, cuda):
    tris = scenes.clustered(1000, seed=2)
    tris[10, 2] = np.inf
    with pytest.raises(kdgb_lib.KdgbError) as e:
        kdgb_lib.KDTree.build(tris)
    assert e.value.status == 6


def test_degenerate_duplicates_error(kdgb_lib, cuda):
    tris = np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (40, 1))
    with pytest.raises(kdgb_lib.KdgbError) as e:
        kdgb_lib.KDTree.build(tris, max_levels=20)
    assert e.value.status == 5


def test_invalid_params(kdgb_lib, cuda):
    tris = scenes.clustered(100, seed=2)
    for bad in (dict(leaf_size=33), dict(leaf_size=0), dict(lower=5), dict(mode=7), dict(split_method=7),
                dict(lower=2, traversal_cost=-1.0)):
        with pytest.raises(kdgb_lib.KdgbError) as e:
            kdgb_lib.KDTree.build(tris, **bad)
        assert e.value.status == 1
    # The reference's SPLIT method throws NotImplemented.
    with pytest.raises(kdgb_lib.KdgbError) as e:
        kdgb_lib.KDTree.build(tris, split_method=2)
    assert e.value.status == 8
