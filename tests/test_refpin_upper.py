"""The oracle's whole build, checked bit for bit against the reference's OWN
kernels.

`oracle/refpin/refpin_upper.cpp` compiles the upper-phase kernels
unmodified with g++ (Utils/CUDA/Kernels/TriangleUpper.h,
TriangleUpperSegment.h, TriangleUpperChildren.h, EmptySpaceSplitting.h and
ReduceSegments.h). It drives them level by level as
TriangleMapUpperCreator.cu does, one thread at a time, with plain prefix sums
for the CUDPP scans. The two reductions that are warp- or barrier-synchronous
(ReduceSegmentsUnrolled, FinalSegmentedReduce) are computed directly: they
compute order-free minima and maxima, which are exact.

Chained with the lower creators of `refpin_lower.cpp`, this reproduces the
reference's build from its own kernels. Every node and reference array the
oracle makes must match it bit for bit. The one exception is the w of the
reduced node boxes, which the reference leaves undefined.

The library is built into oracle/_ref where the reference tree is available.
Elsewhere these tests skip.
"""
import numpy as np
import pytest

from kdgb import scenes


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.refpin_upper_lib() is None or oracle.refpin_lib() is None:
        pytest.skip("the reference tree is not available to compile the pin libraries")
    return oracle


def _scene(name):
    if name == "heightfield":
        return scenes.heightfield(64, 32, seed=1)[0]
    if name == "clustered":
        return scenes.clustered(6000, seed=4)
    if name == "large":
        return scenes.clustered(60000, seed=9)
    rng = np.random.default_rng(7)
    c = rng.random((3000, 1, 3)).astype(np.float32)
    tris = (c + rng.normal(size=(3000, 3, 3)).astype(np.float32) * 0.02).reshape(-1, 9)
    tris[::9, 3:6] = tris[::9, 0:3]  # zero-area triangles
    tris[::13] *= np.float32(40.0)   # a few far-flung ones
    return tris


def _same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)


def _check(got, want, fields):
    assert got.n_nodes == want.n_nodes
    for f in fields:
        a, b = getattr(got, f), getattr(want, f)
        if f in ("aabb_min", "aabb_max"):
            a, b = a[:, :3], b[:, :3]  # w of the reduced boxes is undefined in the reference
        assert _same(a, b), f


UPPER = {
    "box": dict(),
    "divide": dict(split_method=1),
    "no_ess": dict(split_empty_space=0),
    "no_ess_no_propagate": dict(split_empty_space=0, propagate_aabbs=0),
    "threshold_0.2": dict(empty_space_threshold=0.2),
    "threshold_0.6_divide": dict(empty_space_threshold=0.6, split_method=1),
}
UPPER_FIELDS = ("info", "split", "children", "prim_index", "bitmap", "parent", "aabb_min", "aabb_max",
                "prim_indices", "leaf_ids", "prim_min", "prim_max")


@pytest.mark.parametrize("setting", list(UPPER))
@pytest.mark.parametrize("scene", ["heightfield", "clustered", "soup"])
def test_upper_creator_pinned(ref, setting, scene):
    """Upper phase plus the BITMAP leaf conversion: every node, the upper-leaf
    references (their clipped boxes with the triangle id in w) and the leaf
    list."""
    tris = _scene(scene)
    kw = UPPER[setting]
    got, _ = ref.ref_build(tris, lower=0, **kw)
    want = ref.build(tris, lower=0, **kw)
    _check(got, want, UPPER_FIELDS)
    assert got.upper_levels == want.upper_levels
    assert want.n_nodes > 100


@pytest.mark.parametrize("lower,cost,propagate,upper", [
    (1, 24.0, 1, "box"), (1, 1.0, 1, "box"), (1, 1.0, 0, "no_ess"), (1, 24.0, 1, "divide"),
    (2, 24.0, 1, "box"), (2, 16.0, 1, "divide"), (2, 0.0, 0, "no_ess_no_propagate")])
@pytest.mark.parametrize("scene", ["heightfield", "clustered", "soup", "large"])
def test_whole_build_pinned(ref, lower, cost, propagate, upper, scene):
    """Upper creator then the SAH (1) or BALANCED (2) lower creator, all from
    the reference's kernels, against the oracle's whole build."""
    tris = _scene(scene)
    kw = dict(UPPER[upper])
    kw["propagate_aabbs"] = propagate
    got, levels = ref.ref_build(tris, lower=lower, traversal_cost=cost, **kw)
    want = ref.build(tris, lower=lower, traversal_cost=cost, **kw)
    _check(got, want, ("info", "split", "children", "prim_index", "bitmap", "area", "aabb_min", "aabb_max"))
    assert levels == want.lower_levels
    assert _same(got.prim_indices, want.prim_indices) and _same(got.leaf_ids, want.leaf_ids)


def test_settings_change_the_tree(ref):
    """The comparison has teeth: the threshold, the split method and the
    empty-space splits each change the reference's tree."""
    tris = _scene("clustered")
    base, _ = ref.ref_build(tris)
    for kw in (dict(empty_space_threshold=0.2), dict(split_method=1), dict(split_empty_space=0)):
        other, _ = ref.ref_build(tris, **kw)
        assert other.n_nodes != base.n_nodes or not _same(other.split, base.split), kw
