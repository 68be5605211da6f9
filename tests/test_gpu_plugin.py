"""The C++ plugin shims (include/kdgb_plugin.hpp) and the geometry kernels:
OscCUDAMeshNode animation, GeometryList collection (AddMeshKernel) and a
TriangleMap + three tracers frame, checked against numpy and the oracle."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    pytest.fail("CUDA toolkit not found")


def test_cpp_plugin_frame_matches_oracle(kdgb_lib, cuda, oracle, tmp_path):
    cuda_home = _cuda_home()
    libdir = os.path.dirname(kdgb_lib.library_path())
    exe = str(tmp_path / "plugin_demo")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(cuda_home, "include"), os.path.join(HERE, "helpers", "plugin_demo.cpp"),
                    "-L", libdir, "-lkdgb", "-L", os.path.join(cuda_home, "lib64"), "-lcudart",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    out = str(tmp_path / "frame.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.uint8)
    T, n = np.frombuffer(raw[:8].tobytes(), np.int32)
    off = 8
    tris = np.frombuffer(raw[off:off + 36 * T].tobytes(), np.float32).reshape(T, 9); off += 36 * T
    o = np.frombuffer(raw[off:off + 12 * n].tobytes(), np.float32).reshape(n, 3); off += 12 * n
    d = np.frombuffer(raw[off:off + 12 * n].tobytes(), np.float32).reshape(n, 3); off += 12 * n
    res = []
    for _ in range(3):
        h = np.frombuffer(raw[off:off + 4 * n].tobytes(), np.int32); off += 4 * n
        t = np.frombuffer(raw[off:off + 4 * n].tobytes(), np.float32); off += 4 * n
        res.append((h, t))
    nrm = []
    for _ in range(3):
        nrm.append(np.frombuffer(raw[off:off + 16 * T].tobytes(), np.float32).reshape(T, 4)); off += 16 * T
    c0 = raw[off:off + 4 * T].reshape(T, 4); off += 4 * T
    pixels = []
    for _ in range(3):
        pixels.append(raw[off:off + 4 * n].reshape(n, 4)); off += 4 * n
    side = int(round(np.sqrt(n)))
    probes = [(0, 0), (side // 2, side // 3), (side - 1, 17), (5, side - 1)]
    host_traces = []
    for _ in range(3):
        rows = []
        for _ in probes:
            ht = int(np.frombuffer(raw[off:off + 4].tobytes(), np.int32)[0])
            tt = np.frombuffer(raw[off + 4:off + 8].tobytes(), np.float32)[0]
            rows.append((ht, tt, raw[off + 8:off + 12].copy())); off += 12
        host_traces.append(rows)
    assert off == raw.shape[0]
    assert T == 2 * 48 * 48
    tree = oracle.build(tris, lower=1)  # TriangleMap defaults + SetLowerAlgorithm(SAH)
    for (h, t), px, tracer in zip(res, pixels, (0, 1, 2)):
        hr, tr, _, _ = oracle.trace(tree, tris, o, d, tracer=tracer)
        assert np.array_equal(h, hr), tracer
        m = hr >= 0
        assert np.array_equal(t[m].view(np.uint32), tr[m].view(np.uint32))
        assert m.mean() > 0.5
        want = oracle.trace_shaded(tree if tracer != 2 else None, tris, o, d, nrm[0], nrm[1], nrm[2], c0,
                                   tracer=tracer)
        assert np.array_equal(px, want), tracer
        assert (px[m, 3] > 0).all()
        # HostTrace(x, y) re-traces pixel x + y * side on the device: the same
        # first hit and colour as the full frame.
        for (x, y), (ht, tt, rgba) in zip(probes, host_traces[tracer]):
            i = x + y * side
            assert ht == hr[i], (tracer, x, y)
            if hr[i] >= 0:
                assert np.float32(tt).view(np.uint32) == tr[i].view(np.uint32)
            assert np.array_equal(rgba, want[i]), (tracer, x, y)


def test_geometry_gather_matches_numpy(kdgb_lib, cuda):
    import torch
    from kdgb import _lib
    V = 500
    verts = np.concatenate([np.stack([scenes.uniform(3, V, k) for k in range(3)], 1),
                            np.ones((V, 1))], 1).astype(np.float32)
    idx = (scenes.uniform(4, 3 * 700, 0) * V).astype(np.uint32)
    idx[17] = V + 5  # out of range: that triangle becomes NaN
    M = np.array([[0.9, 0.1, 0.0, 0.5], [-0.1, 0.9, 0.2, 0.25], [0.0, -0.2, 1.1, 0.5], [0, 0, 0, 1]], np.float32)
    vd = torch.from_numpy(verts).cuda()
    idd = torch.from_numpy(idx.view(np.int32)).cuda()
    out = torch.empty((700, 9), dtype=torch.float32, device="cuda")
    Mh = np.ascontiguousarray(M.reshape(-1))
    _lib.check(_lib.lib().kdgb_geometry_gather(C.c_void_p(vd.data_ptr()), V, C.c_void_p(idd.data_ptr()), 2100,
                                              Mh.ctypes.data_as(C.c_void_p), C.c_void_p(out.data_ptr()), None),
               "gather")
    got = out.cpu().numpy()
    safe = np.minimum(idx, V - 1).astype(np.int64)
    vv = verts[safe]
    ref = np.zeros((2100, 3), np.float32)
    for r in range(3):
        s = (M[r, 0] * vv[:, 0]).astype(np.float32)
        for c in range(1, 4):
            s = (s + (M[r, c] * vv[:, c]).astype(np.float32)).astype(np.float32)
        ref[:, r] = s
    ref = ref.reshape(700, 9)
    bad = np.zeros(700, bool)
    bad[17 // 3] = True
    assert np.isnan(got[bad]).any() and not np.isnan(got[~bad]).any()
    assert np.array_equal(got[~bad], ref[~bad])


def test_osc_update_surface(kdgb_lib, cuda):
    import torch
    from kdgb import _lib
    detail, height, time = 20, 0.1, 1.25
    d = detail + 1
    i, j = np.meshgrid(np.arange(d), np.arange(d), indexing="xy")
    verts = np.stack([i.ravel() * 0.1, np.full(d * d, height), j.ravel() * 0.1, np.ones(d * d)], 1).astype(np.float32)
    vd = torch.from_numpy(verts).cuda()
    nd = torch.zeros_like(vd)
    _lib.check(_lib.lib().kdgb_osc_update_surface(C.c_void_p(vd.data_ptr()), C.c_void_p(nd.data_ptr()), detail,
                                                 height, time, None), "osc")
    v, n = vd.cpu().numpy(), nd.cpu().numpy()
    x = (np.arange(d * d) % d).astype(np.float32)
    y = (np.arange(d * d) // d).astype(np.float32)
    ax = np.float32(0.3) * x + np.float32(time)
    ay = np.float32(0.3) * y + np.float32(time)
    ey = np.float32(height) + np.float32(0.2) * np.cos(ax) + np.float32(0.2) * np.sin(ay)
    # detail = 20 is not a multiple of 16, so every vertex is updated.
    assert np.allclose(v[:, 1], ey, atol=2e-6)
    assert np.array_equal(v[:, [0, 2, 3]], verts[:, [0, 2, 3]])
    nx = -0.2 * np.sin(ax) * 0.3
    nz = 0.2 * np.cos(ay) * 0.3
    assert np.allclose(n[:, 0], nx, atol=2e-6) and np.allclose(n[:, 2], nz, atol=2e-6)
    assert np.allclose(n[:, 1], 1 - nx * nx - nz * nz, atol=2e-6)


def test_osc_update_keeps_reference_grid_quirk(kdgb_lib, cuda):
    # OscCUDAMeshNode.cu sizes its grid from `detail`: with detail = 16 the
    # last row and column (index 16) keep their heights.
    import torch
    from kdgb import _lib
    detail = 16
    d = detail + 1
    verts = np.zeros((d * d, 4), np.float32)
    verts[:, 1] = 7.0
    vd = torch.from_numpy(verts).cuda()
    nd = torch.zeros_like(vd)
    _lib.check(_lib.lib().kdgb_osc_update_surface(C.c_void_p(vd.data_ptr()), C.c_void_p(nd.data_ptr()), detail,
                                                 0.0, 0.5, None), "osc")
    v = vd.cpu().numpy().reshape(d, d, 4)
    assert (v[16, :, 1] == 7.0).all() and (v[:, 16, 1] == 7.0).all() and (v[:16, :16, 1] != 7.0).all()
