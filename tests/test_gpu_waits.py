"""Bounded device-side waits give up cleanly.

The look-back scans (every build level) wait for a predecessor tile's
status.  kdgb_check_scan_giveup runs one such wait on a tile whose
predecessor never publishes -- a flag that nothing sets -- with a small poll
limit: the wait must stop, record KDGB_ERR_TIMEOUT, finish its tile with the
missing prefix counted as 0, and leave the device usable.  No fault, trap or
unbounded wait is involved."""
import ctypes as C

import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("spin_limit", [1, 64, 4096])
def test_lookback_wait_gives_up_with_timeout(kdgb_lib, cuda, spin_limit):
    from kdgb import _lib
    status, prefix = C.c_int32(-1), C.c_int32(-1)
    _lib.check(_lib.lib().kdgb_check_scan_giveup(spin_limit, C.byref(status), C.byref(prefix),
                                                 C.c_void_p(cuda.cuda.current_stream().cuda_stream)),
               "kdgb_check_scan_giveup")
    assert status.value == _lib.ERR_TIMEOUT
    assert prefix.value == 0
    # The context is intact: a build and a trace still run and agree with
    # brute force.
    tris = scenes.clustered(3000, seed=9)
    o, d = scenes.camera_rays(32, 32)
    with kdgb_lib.KDTree.build(tris) as tree:
        h = tree.trace(o, d)[0].cpu().numpy()
    hb = kdgb_lib.trace_brute(tris, o, d)[0].cpu().numpy()
    assert np.array_equal(h, hb)


def test_giveup_check_rejects_bad_limit(kdgb_lib, cuda):
    from kdgb import _lib
    status, prefix = C.c_int32(), C.c_int32()
    rc = _lib.lib().kdgb_check_scan_giveup(0, C.byref(status), C.byref(prefix), None)
    assert rc == _lib.ERR_INVALID_ARGUMENT
