"""kdgb_trace_brute_noalloc: brute-force tracing for callers that cannot
allocate device memory while they run (a frame loop that must not stall on
cudaMalloc, or a host whose own allocator already holds the device memory).

The entry point keeps its scratch in a fixed array inside the library, so it
must give the same answer as kdgb_trace_brute, call after call, even though
every call reuses (and overwrites) that one array.  This file is collected
last so a failure here never hides the result of another test.
"""
import ctypes as C

import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def _noalloc(kdgb_lib, tris, o, d, tie=0):
    import torch
    from kdgb import _lib
    tri = torch.from_numpy(np.ascontiguousarray(tris, np.float32)).cuda()
    od = torch.from_numpy(np.ascontiguousarray(o, np.float32)).cuda()
    dd = torch.from_numpy(np.ascontiguousarray(d, np.float32)).cuda()
    n = od.shape[0]
    hit = torch.empty(n, dtype=torch.int32, device="cuda")
    t, u, v = (torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = _lib.lib().kdgb_trace_brute_noalloc(C.c_void_p(tri.data_ptr()), tri.shape[0], tie,
                                            C.c_void_p(od.data_ptr()), C.c_void_p(dd.data_ptr()), n,
                                            C.c_void_p(hit.data_ptr()), C.c_void_p(t.data_ptr()),
                                            C.c_void_p(u.data_ptr()), C.c_void_p(v.data_ptr()), stream)
    _lib.check(rc, "kdgb_trace_brute_noalloc")
    torch.cuda.synchronize()
    return tuple(x.cpu().numpy() for x in (hit, t, u, v))


def _compare(got, ref):
    h, t, u, v = got
    hr, tr, ur, vr = (x.cpu().numpy() for x in ref)
    assert np.array_equal(h, hr)
    m = hr >= 0
    for a, b in ((t, tr), (u, ur), (v, vr)):
        assert np.allclose(a[m], b[m], rtol=RTOL, atol=0)
    assert np.isinf(t[~m]).all()


def test_noalloc_matches_brute_on_two_calls_in_a_row(kdgb_lib, cuda):
    # First call: 3000 triangles; second call: 256, so stale records from the
    # first call sit past the end of the second call's triangles.
    big = scenes.clustered(3000, seed=31)
    lo, hi = big.reshape(-1, 3).min(0), big.reshape(-1, 3).max(0)
    o1, d1 = scenes.random_rays(4096, 32, lo, hi)
    small = scenes.heightfield(16, 8, seed=1)[0]
    o2, d2 = scenes.camera_rays(64, 64)
    for tris, o, d in ((big, o1, d1), (small, o2, d2)):
        ref = kdgb_lib.trace_brute(tris, o, d)
        got = _noalloc(kdgb_lib, tris, o, d)
        _compare(got, ref)
        assert (got[0] >= 0).sum() > 100


def test_noalloc_rejects_too_many_triangles(kdgb_lib, cuda):
    from kdgb import _lib
    import torch
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = _lib.lib().kdgb_trace_brute_noalloc(C.c_void_p(buf.data_ptr()), _lib.NOALLOC_MAX_TRIS + 1, 0,
                                            C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), 1,
                                            C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()),
                                            C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), None)
    assert rc == _lib.ERR_CAPACITY
    assert b"exceeds the static scratch" in _lib.lib().kdgb_last_error()
