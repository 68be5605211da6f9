"""Autotuner (kdgb_autotune): picks from its candidate sets, never returns a
choice worse than the starting parameters it measured, and its choice is a
parameter set whose tree and trace still match the oracle bit for bit."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)


def test_autotune_single_mesh(kdgb_lib, cuda, oracle):
    tris = scenes.clustered(30000, seed=21)
    o, d = scenes.camera_rays(128, 96)
    bp = kdgb_lib.build_params(mode=1, upper_levels=8, **SAH_C1)
    tp = kdgb_lib.trace_params(tracer=1, stack_depth=4)
    r = kdgb_lib.autotune(tris, o, d, build=bp, trace=tp, builds_per_trace=1.0, reps=2)
    assert r.trials >= 7
    assert r.objective <= r.baseline
    assert r.build.leaf_size in (16, 24, 32)
    assert r.build.sah_bins in (8, 16, 32)
    assert r.trace.stack_depth in (2, 4, 8)
    assert r.trace.block_size in (0, 64, 128, 256)
    assert r.build.max_levels == bp.max_levels
    kw = dict(mode=1, upper_levels=8, leaf_size=r.build.leaf_size, sah_bins=r.build.sah_bins, **SAH_C1)
    ref = oracle.build(tris, **kw)
    with kdgb_lib.KDTree.build(tris, r.build) as tree:
        h = tree.trace(o, d, r.trace)[0].cpu().numpy()
    hr, _, _, _ = oracle.trace(ref, tris, o, d, tracer=1, stack_depth=r.trace.stack_depth)
    assert np.array_equal(h, hr)


def test_autotune_batch_build_only(kdgb_lib, cuda):
    sizes = [2000, 500, 9000]
    tris = np.concatenate([scenes.clustered(s, seed=30 + i) for i, s in enumerate(sizes)])
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    r = kdgb_lib.autotune(tris, mesh_offsets=off, reps=1)
    assert r.objective <= r.baseline and r.trace_ms < 0.05  # no rays: an empty timed region
    assert r.build.leaf_size in (16, 24, 32)


def test_autotune_rejects_bad_arguments(kdgb_lib, cuda):
    tris = scenes.clustered(1000, seed=31)
    with pytest.raises(kdgb_lib.KdgbError):
        kdgb_lib.autotune(tris, reps=0)
    with pytest.raises(kdgb_lib.KdgbError):
        kdgb_lib.autotune(tris, mesh_offsets=np.array([0, 10]), reps=1)  # offsets must cover every triangle
