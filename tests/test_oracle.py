"""CPU tests of the oracle: known answers for the intersection primitive,
the reference's CPU_VERIFY invariants on built trees, tie rules and
agreement between the three tracers."""
import numpy as np
import pytest

from kdgb import scenes


def tri_soup(n, seed, scale=0.05):
    """Random small triangles in the unit cube."""
    c = np.stack([scenes.uniform(seed, n, k) for k in range(3)], axis=1)
    off = (np.stack([scenes.uniform(seed, n, 10 + k) for k in range(9)], axis=1) - 0.5) * scale
    return np.ascontiguousarray((np.tile(c, 3) + off).astype(np.float32))


# ---------------------------------------------------------------------------
# Moeller-Trumbore known answers (IRayTracer.h:111-145)
# ---------------------------------------------------------------------------

def test_mt_center_hit(oracle):
    hit, tuv = oracle.moeller_trumbore([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.25, 0.25, 1], [0, 0, -1])
    assert hit
    assert tuv.tolist() == [1.0, 0.25, 0.25]


def test_mt_edges_inclusive(oracle):
    # u + v == 1 exactly on the hypotenuse is a hit (<= 1), u == 0 is a hit.
    hit, tuv = oracle.moeller_trumbore([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 2], [0, 0, -1])
    assert hit and tuv[0] == 2.0 and tuv[1] + tuv[2] == 1.0
    hit, tuv = oracle.moeller_trumbore([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.0, 0.5, 2], [0, 0, -1])
    assert hit and tuv[1] == 0.0


def test_mt_rejections(oracle):
    tri = ([0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert not oracle.moeller_trumbore(*tri, [0.6, 0.6, 1], [0, 0, -1])[0]      # outside
    assert not oracle.moeller_trumbore(*tri, [0.2, 0.2, 1], [1, 0, 0])[0]       # parallel (det = 0)
    assert not oracle.moeller_trumbore(*tri, [0.2, 0.2, -1], [0, 0, -1])[0]     # behind (t < 0)
    assert not oracle.moeller_trumbore(*tri, [0.2, 0.2, 1], [0, 0, -1], 0.5)[0]  # beyond t_max
    assert oracle.moeller_trumbore(*tri, [0.2, 0.2, 1], [0, 0, -1], 1.0)[0]      # t == t_max accepted


# ---------------------------------------------------------------------------
# Tree invariants (TriangleMapUpperCreator.cu:761-902 CPU_VERIFY checks)
# ---------------------------------------------------------------------------

def check_tree(tree, tris, leaf_size=32):
    n = tree.n_nodes
    info, ch, bm, pi = tree.info, tree.children, tree.bitmap, tree.prim_index
    # Every node reachable exactly once from the root (a tree, not a DAG).
    seen = np.zeros(n, np.int32)
    stack = [0]
    while stack:
        k = stack.pop()
        seen[k] += 1
        if info[k] != 0:
            stack += [int(ch[k, 0]), int(ch[k, 1])]
    assert (seen == 1).all()
    assert set(np.unique(info)) <= {0, 1, 2, 3}
    leaves = np.nonzero(info == 0)[0]
    nref = tree.prim_indices.shape[0]
    for k in leaves:
        b = np.uint32(bm[k])
        if b:
            top = 31 - int(np.log2(int(b)))
            assert 0 <= pi[k] and pi[k] + (31 - top) < nref
    # Every reference id is a valid triangle.
    assert ((tree.prim_indices >= 0) & (tree.prim_indices < tris.shape[0])).all()
    # Clipped reference boxes lie inside their triangle's box (CPU_VERIFY 3).
    v = tris.reshape(-1, 3, 3)
    tmin, tmax = v.min(1), v.max(1)
    ids = tree.prim_indices
    assert (tree.prim_min[:, :3] >= tmin[ids]).all() and (tree.prim_max[:, :3] <= tmax[ids]).all()
    # Each triangle appears in at least one leaf (no triangle is lost).
    used = np.zeros(tris.shape[0], bool)
    for k in leaves:
        b = int(np.uint32(bm[k]))
        i = 0
        while b:
            if b & 1:
                used[ids[pi[k] + i]] = True
            b >>= 1
            i += 1
    area = np.linalg.norm(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), axis=1)
    return used, area


@pytest.mark.parametrize("lower", [0, 1, 2])
@pytest.mark.parametrize("scene", ["heightfield", "clustered", "soup"])
def test_tree_invariants(oracle, scene, lower):
    if scene == "heightfield":
        tris = scenes.heightfield(32, 16, seed=1)[0]
    elif scene == "clustered":
        tris = scenes.clustered(3000, seed=4)
    else:
        tris = tri_soup(2000, 7)
    tree = oracle.build(tris, lower=lower)
    used, area = check_tree(tree, tris)
    if lower != 1:
        assert used.all()
    else:
        # The SAH lower phase drops zero-area triangles (LowerTriangleMap.h:74).
        assert used[area > 0].all()


@pytest.mark.parametrize("upper", [0, 4, 8])
def test_tuned_tree_invariants_and_hits(oracle, upper):
    tris = scenes.clustered(20000, seed=17)
    kw = dict(mode=1, upper_levels=upper, lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
    tree = oracle.build(tris, **kw)
    used, area = check_tree(tree, tris)
    assert used[area > 0].all()
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    o, d = scenes.random_rays(3000, 18, lo, hi)
    hb = oracle.trace(None, tris, o, d, tracer=2)[0]
    for tracer in (0, 1):
        assert (oracle.trace(tree, tris, o, d, tracer=tracer)[0] == hb).mean() >= 0.999


def test_tuned_differs_from_reference_below_median_levels(oracle):
    tris = scenes.clustered(20000, seed=19)
    a = oracle.build(tris, mode=1, upper_levels=8)
    b = oracle.build(tris)
    assert a.n_nodes != b.n_nodes or not np.array_equal(a.split, b.split)
    c = oracle.build(tris, mode=1, upper_levels=64)  # never reaches the SAH levels
    assert np.array_equal(c.split, b.split) and np.array_equal(c.children, b.children)


def popc(x):
    return bin(int(np.uint32(x))).count("1")


@pytest.mark.parametrize("cost", [0.0, 16.0, 24.0])
def test_balanced_split_rule(oracle, cost):
    """Every balanced split divides a node's reference set into two covering
    subsets with (cost + small^2 + large^2) / n < n (LowerTriangleMap.h:
    299-369); every lower leaf has no plane that passes the rule."""
    tris = scenes.clustered(4000, seed=21)
    tree = oracle.build(tris, lower=2, traversal_cost=cost)
    assert tree.lower_levels > 1
    splits = 0
    stack = [int(k) for k in tree.leaf_ids]
    while stack:
        k = stack.pop()
        if tree.info[k] == 0:
            continue
        l, r = (int(c) for c in tree.children[k])
        b, bl, br = (int(np.uint32(tree.bitmap[j])) for j in (k, l, r))
        assert tree.prim_index[l] == tree.prim_index[r] == tree.prim_index[k]
        assert bl | br == b and bl & ~b == 0 and br & ~b == 0
        n, a, c = popc(b), popc(bl), popc(br)
        assert np.float32(cost + (a * a + c * c)) / np.float32(n) < n
        assert max(a, c) < n
        splits += 1
        stack += [l, r]
    assert splits > 0
    # Balanced trees keep every triangle and trace like brute force.
    used, _ = check_tree(tree, tris)
    assert used.all()
    assert (tree.area == 0).all()


@pytest.mark.parametrize("lower", [0, 2])
def test_divide_keeps_triangles_and_traces_exactly(oracle, lower):
    """DIVIDE (TriangleUpperChildren.h:64-142) drops references whose
    triangle misses a half box, but never a triangle from every leaf: kd
    traversal of the tree equals brute force."""
    tris = tri_soup(6000, 23, scale=0.1)
    box = oracle.build(tris, lower=lower)
    div = oracle.build(tris, lower=lower, split_method=1)
    assert div.prim_indices.shape[0] < box.prim_indices.shape[0]
    used, _ = check_tree(div, tris)
    assert used.all()
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    o, d = scenes.random_rays(4000, 24, lo, hi)
    hb, tb, _, _ = oracle.trace(None, tris, o, d, tracer=2)
    for tracer in (0, 1):
        h, t, _, _ = oracle.trace(div, tris, o, d, tracer=tracer)
        assert np.array_equal(h, hb)
        if tracer == 0:
            assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))
        else:  # the short stack measures t from a moved origin
            assert np.allclose(t, tb, rtol=1e-5)


def test_split_method_and_lower_validation(oracle):
    tris = scenes.clustered(200, seed=2)
    for bad in (dict(split_method=2), dict(lower=3), dict(lower=2, traversal_cost=-1.0)):
        with pytest.raises(RuntimeError, match="invalid argument"):
            oracle.build(tris, **bad)


def test_upper_leaf_boxes_contain_references(oracle):
    tris = scenes.clustered(3000, seed=9)
    tree = oracle.build(tris)
    for k in tree.leaf_ids:
        a, n = int(tree.prim_index[k]), bin(int(np.uint32(tree.bitmap[k]))).count("1")
        if n == 0:
            continue
        lo, hi = tree.aabb_min[k, :3], tree.aabb_max[k, :3]
        assert (tree.prim_min[a:a + n, :3] >= lo).all() and (tree.prim_max[a:a + n, :3] <= hi).all()


def test_build_deterministic(oracle):
    tris = scenes.clustered(5000, seed=11)
    a, b = oracle.build(tris, lower=1), oracle.build(tris, lower=1)
    for f in ("info", "split", "children", "bitmap", "prim_index", "prim_indices", "aabb_min", "aabb_max"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_empty_and_tiny_scenes(oracle):
    empty = np.zeros((0, 9), np.float32)
    tree = oracle.build(empty)
    # The root is always split (TriangleMapUpperCreator.cu:139-161): an x split
    # of the +-fInfinity box at 0 with two empty leaves.
    assert tree.n_nodes == 3 and tree.info.tolist() == [1, 0, 0] and (tree.bitmap[1:] == 0).all()
    o, d = scenes.camera_rays(8, 8)
    h, t, u, v = oracle.trace(tree, empty, o, d)
    assert (h == -1).all() and np.isinf(t).all()
    one = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    tree = oracle.build(one)
    h, t, _, _ = oracle.trace(tree, one, [[0.2, 0.2, 1]], [[0, 0, -1]])
    assert h[0] == 0 and t[0] == 1.0


def test_nonfinite_rejected(oracle):
    tris = scenes.clustered(100, seed=1)
    tris[5, 4] = np.nan
    with pytest.raises(RuntimeError, match="non-finite"):
        oracle.build(tris)


def test_degenerate_duplicates_terminate(oracle):
    # 40 identical triangles cannot be separated by any plane: the upper loop
    # must stop at max_levels with an error instead of running forever.
    tris = np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (40, 1))
    with pytest.raises(RuntimeError, match="max_levels"):
        oracle.build(tris, max_levels=20)


# ---------------------------------------------------------------------------
# Tracers
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("tracer", [0, 1])
@pytest.mark.parametrize("lower", [0, 1, 2])
def test_kd_tracers_match_brute_force(oracle, tracer, lower):
    tris = scenes.clustered(4000, seed=12)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    o, d = scenes.random_rays(3000, 13, lo, hi)
    tree = oracle.build(tris, lower=lower)
    hb, tb, ub, vb = oracle.trace(None, tris, o, d, tracer=2)
    h, t, u, v = oracle.trace(tree, tris, o, d, tracer=tracer)
    assert (h == hb).mean() >= 0.999
    same = (h == hb) & (h >= 0)
    assert np.allclose(t[same], tb[same], rtol=1e-6)


def test_f64_error_is_small(oracle):
    tris = scenes.heightfield(64, 32, seed=1)[0]
    o, d = scenes.camera_rays(128, 128)
    h, t, u, v = oracle.trace(None, tris, o, d, tracer=2)
    hf, tf, uf, vf = oracle.trace_brute_f64(tris, o, d)
    agree = (h == hf) & (h >= 0)
    assert agree.sum() > 1000
    assert np.max(np.abs(t[agree] - tf[agree]) / tf[agree]) < 1e-5


def test_tie_rules_on_duplicates(oracle):
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    tris = np.stack([tri, tri, tri])
    o, d = [[0.2, 0.2, 1.0]], [[0, 0, -1]]
    assert oracle.trace(None, tris, o, d, tracer=2, tie=oracle.TIE_LOWEST_ID)[0][0] == 0
    assert oracle.trace(None, tris, o, d, tracer=2, tie=oracle.TIE_REF_LAST)[0][0] == 2
    tree = oracle.build(tris)
    assert oracle.trace(tree, tris, o, d, tracer=0, tie=oracle.TIE_LOWEST_ID)[0][0] == 0
    assert oracle.trace(tree, tris, o, d, tracer=0, tie=oracle.TIE_REF_LAST)[0][0] == 2


def test_shared_edge_tie(oracle):
    # Two triangles sharing the edge x + y = 1; a ray exactly through the
    # edge hits both at t = 1; the lowest id wins by default.
    tris = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0], [1, 1, 0, 0, 1, 0, 1, 0, 0]], np.float32)
    o, d = [[0.5, 0.5, 1.0]], [[0, 0, -1]]
    hit, t, _, _ = oracle.trace(None, tris, o, d, tracer=2)
    assert hit[0] == 0 and t[0] == 1.0
    assert oracle.trace(None, tris, o, d, tracer=2, tie=oracle.TIE_REF_LAST)[0][0] == 1


def test_zero_direction_components(oracle):
    tris = scenes.heightfield(16, 16, seed=2)[0]
    tree = oracle.build(tris)
    o = np.array([[0.3, 0.3, 2.0], [0.7, 0.2, 2.0], [0.3, 0.3, 2.0]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, -1], [1, 0, 0]], np.float32)
    for tracer in (0, 1):
        h, t, _, _ = oracle.trace(tree, tris, o, d, tracer=tracer)
        assert h[0] >= 0 and h[1] >= 0 and h[2] == -1


def test_stack_depths_agree(oracle):
    tris = scenes.clustered(3000, seed=21)
    tree = oracle.build(tris)
    o, d = scenes.camera_rays(48, 48)
    ref = oracle.trace(tree, tris, o, d, tracer=0)[0]
    for depth in (1, 2, 4, 8):
        h = oracle.trace(tree, tris, o, d, tracer=1, stack_depth=depth)[0]
        assert (h == ref).mean() >= 0.999


def shadow_scene():
    """A flat 32x32 ground grid at z = 0.5 and an 8x8 occluder grid over
    [0.3, 0.5]^2 at z = 0.8."""
    ground = scenes.heightfield(32, 32, seed=1, amplitude=0.0)[0]
    occ = scenes.heightfield(8, 8, seed=1, amplitude=0.0)[0].reshape(-1, 3, 3).copy()
    occ[..., :2] = 0.3 + 0.2 * occ[..., :2]
    occ[..., 2] = 0.8
    return np.ascontiguousarray(np.concatenate([ground, occ.reshape(-1, 9)]).astype(np.float32))


def test_shadow_rays(oracle):
    tris = shadow_scene()
    tree = oracle.build(tris)
    pts = np.array([[0.4, 0.4, 0.5], [0.9, 0.9, 0.5], [0.1, 0.8, 0.5]], np.float32)
    occ = oracle.trace_shadow(tree, tris, pts, (0.4, 0.4, 3.0))
    assert occ.tolist() == [1, 0, 0]


def test_kpow_restatement_accuracy(oracle):
    """The specular power restated from series stays within 2e-5 relative
    of the exact power over the shading loop's range (the fp32 rounding of
    y * log2(x) dominates at large exponents)."""
    import math
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.random(2000).astype(np.float32), np.float32([1e-30, 1e-6, 0.5, 0.999999])])
    for y in (1.0, 2.5, 64.0, 127.5, 128.0):
        for x in xs:
            got = oracle.kpow(float(x), y)
            want = math.pow(float(x), y)
            if want < 1e-30:
                assert got < 1e-29
            else:
                assert abs(got - want) <= 2e-5 * want + 1e-37, (x, y, got, want)
    assert oracle.kpow(0.0, 3.0) == 0.0 and oracle.kpow(0.3, 0.0) == 1.0 and oracle.kpow(1.0, 5.0) == 1.0


def test_shaded_oracle_tracers_agree(oracle):
    """kd-restart and short-stack shade identically (same hits, same
    directions after the reference's inversions) on a small box."""
    from kdgb import scenes
    tris, n0, n1, n2, c0 = scenes.shaded_box(8, 4, seed=2)
    o, d = scenes.camera_rays(32, 16)
    ref = oracle.build(tris)
    a = oracle.trace_shaded(ref, tris, o, d, n0, n1, n2, c0, tracer=0)
    b = oracle.trace_shaded(ref, tris, o, d, n0, n1, n2, c0, tracer=1)
    assert (a[:, 3] > 0).any()
    # the two kd tracers may differ by the short stack's double inversion
    # of the direction; nearly every pixel must agree
    assert (a == b).all(axis=1).mean() > 0.95
