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
    """Hit ids equal; t, u, v equal bit for bit (the arithmetic is the same
    as the allocating entry point's and the oracle's), which also holds them
    within the 1e-6 relative tolerance of the other tests."""
    h, t, u, v = got
    hr, tr, ur, vr = (x.cpu().numpy() if hasattr(x, "cpu") else x for x in ref)
    assert np.array_equal(h, hr), f"{(h != hr).sum()} hit ids differ"
    m = hr >= 0
    for a, b in ((t, tr), (u, ur), (v, vr)):
        assert np.allclose(a[m], b[m], rtol=RTOL, atol=0)
        assert np.array_equal(a[m].view(np.uint32), b[m].view(np.uint32))
    assert np.isinf(t[~m]).all()


def test_noalloc_matches_brute_on_two_calls_in_a_row(kdgb_lib, cuda, oracle):
    # First call: 3000 triangles; second call: 256, so stale records from the
    # first call sit past the end of the second call's triangles.  Each call
    # is checked against the allocating entry point and against the oracle.
    big = scenes.clustered(3000, seed=31)
    lo, hi = big.reshape(-1, 3).min(0), big.reshape(-1, 3).max(0)
    o1, d1 = scenes.random_rays(4096, 32, lo, hi)
    small = scenes.heightfield(16, 8, seed=1)[0]
    o2, d2 = scenes.camera_rays(64, 64)
    for tris, o, d in ((big, o1, d1), (small, o2, d2)):
        got = _noalloc(kdgb_lib, tris, o, d)
        _compare(got, kdgb_lib.trace_brute(tris, o, d))
        _compare(got, oracle.trace(None, tris, o, d, tracer=2))
        assert (got[0] >= 0).sum() > 100


@pytest.mark.parametrize("tie", [0, 1])
def test_noalloc_equal_t_ties(kdgb_lib, cuda, oracle, tie):
    """Every triangle twice (ids i and i + T): each hit is an exact tie, won
    by the lower id (LOWEST_ID) or by the last one tested (REF_LAST)."""
    base = scenes.heightfield(16, 8, seed=4)[0]
    tris = np.concatenate([base, base])
    o, d = scenes.camera_rays(48, 48)
    got = _noalloc(kdgb_lib, tris, o, d, tie=tie)
    _compare(got, oracle.trace(None, tris, o, d, tracer=2, tie=tie))
    _compare(got, kdgb_lib.trace_brute(tris, o, d, tie=tie))
    h = got[0][got[0] >= 0]
    assert h.size > 100
    T = base.shape[0]
    assert ((h < T) if tie == 0 else (h >= T)).all()


def test_noalloc_without_triangles_misses(kdgb_lib, cuda):
    o, d = scenes.camera_rays(16, 16)
    h, t, u, v = _noalloc(kdgb_lib, np.zeros((0, 9), np.float32), o, d)
    assert (h == -1).all() and np.isinf(t).all() and (u == 0).all() and (v == 0).all()


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
