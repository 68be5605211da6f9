"""Shaded trace (kdgb_trace_shaded): the reference's shading loop (hit,
Phong light, reflection, front-to-back blending until alpha 0.97) into an
RGBA8 buffer, bit for bit the CPU restatement's pixels for the three
tracers."""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)


@pytest.mark.parametrize("tracer", [0, 1, 2])
def test_shaded_matches_oracle(kdgb_lib, cuda, oracle, tracer):
    tris, n0, n1, n2, c0 = scenes.shaded_box(32, 16, seed=3)
    o, d = scenes.camera_rays(96, 64)
    ref = oracle.build(tris, **SAH_C1)
    want = oracle.trace_shaded(ref if tracer != 2 else None, tris, o, d, n0, n1, n2, c0, tracer=tracer,
                               stack_depth=4)
    with kdgb_lib.KDTree.build(tris, **SAH_C1) as tree:
        got = tree.trace_shaded(o, d, n0, n1, n2, c0, tracer=tracer, stack_depth=4).cpu().numpy()
    assert np.array_equal(got, want), int((got != want).any(axis=1).sum())
    # the scene makes rays bounce: some pixels are neither empty nor opaque after one hit
    assert (want[:, 3] > 0).mean() > 0.5
    assert len(np.unique(want[:, 3])) > 3


def test_shaded_packets_and_light(kdgb_lib, cuda, oracle):
    tris, n0, n1, n2, c0 = scenes.shaded_box(16, 8, seed=4)
    o, d = scenes.camera_rays(64, 32)
    L = dict(position=(0.5, 0.5, 3.0), ambient=(0.1, 0.1, 0.1), diffuse=(0.8, 0.7, 0.6), specular=(0.5, 0.5, 0.5))
    ref = oracle.build(tris)
    want = oracle.trace_shaded(ref, tris, o, d, n0, n1, n2, c0, light_params=oracle.light(**L), max_bounces=3,
                               tracer=1)
    with kdgb_lib.KDTree.build(tris) as tree:
        got = tree.trace_shaded(o, d, n0, n1, n2, c0, light_params=kdgb_lib.light(**L), max_bounces=3, tracer=1,
                                tile_width=64).cpu().numpy()
    assert np.array_equal(got, want)


def test_gather_attributes(kdgb_lib, cuda):
    import ctypes as C
    import torch
    verts = scenes.heightfield_vertices(8, 4, seed=2)
    idx = scenes.grid_indices(8, 4)
    vn = torch.from_numpy(scenes.vertex_normals(verts, idx)).cuda()
    cols = torch.from_numpy((np.arange(vn.shape[0] * 4) % 251).astype(np.uint8).reshape(-1, 4)).cuda()
    ib = torch.from_numpy(idx.astype(np.int32)).cuda()
    T = idx.shape[0] // 3
    n0, n1, n2 = (torch.empty((T, 4), dtype=torch.float32, device="cuda") for _ in range(3))
    c0 = torch.empty((T, 4), dtype=torch.uint8, device="cuda")
    rot = np.array([0, -1, 0, 1, 0, 0, 0, 0, 1], np.float32)  # 90 degrees about z
    L = kdgb_lib.lib()
    p = lambda t: C.c_void_p(t.data_ptr())
    kdgb_lib.check(L.kdgb_geometry_gather_attributes(p(vn), p(cols), vn.shape[0], p(ib), idx.shape[0],
                                                     rot.ctypes.data_as(C.c_void_p), p(n0), p(n1), p(n2), p(c0),
                                                     C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "gather")
    t = idx.reshape(-1, 3).astype(np.int64)
    vnh = vn.cpu().numpy()
    for k, nk in enumerate((n0, n1, n2)):
        src = vnh[t[:, k]]
        want = np.stack([-src[:, 1], src[:, 0], src[:, 2], np.zeros(T, np.float32)], axis=1)
        assert np.array_equal(nk.cpu().numpy(), want)
    assert np.array_equal(c0.cpu().numpy(), cols.cpu().numpy()[t[:, 0]])
