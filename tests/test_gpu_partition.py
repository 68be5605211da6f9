"""SM partitions (kdgb_sm_partition_*): streams whose kernels keep to a share
of the device's SMs.  A rebuild graph captured on a partition stream and a
trace on the other partition give the same tree and hits as on the whole
device."""
import numpy as np
import pytest
import torch

from kdgb import scenes

pytestmark = pytest.mark.gpu


def test_partition_sizes(kdgb_lib, cuda):
    total = torch.cuda.get_device_properties(0).multi_processor_count
    with kdgb_lib.SmPartition(32) as part:
        a, b = part.sms(0), part.sms(1)
        assert a >= 32 and b >= 1 and a + b <= total


def test_partition_rejects_bad_sizes(kdgb_lib, cuda):
    total = torch.cuda.get_device_properties(0).multi_processor_count
    for bad in (0, -4, total):
        with pytest.raises(kdgb_lib.KdgbError):
            kdgb_lib.SmPartition(bad)


def test_graph_and_trace_on_partitions(kdgb_lib, cuda, oracle):
    kw = dict(mode=1, upper_levels=8, sah_bins=32, lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
    tris = scenes.clustered(20000, seed=41)
    o, d = scenes.camera_rays(128, 96)
    ref = oracle.build(tris, **kw)
    td = torch.from_numpy(tris).cuda()
    od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    tp = kdgb_lib.trace_params(tracer=kdgb_lib.TRACER_SHORTSTACK, stack_depth=8, tile_width=128)
    with kdgb_lib.KDTree.build(td, **kw) as whole:
        want = [x.cpu().numpy() for x in whole.trace_primary_shadow(od, dd, (0.5, 3.0, 0.5), tp)]
    with kdgb_lib.SmPartition(32) as part:
        build_s, trace_s = part.stream(0), part.stream(1)
        tree = kdgb_lib.KDTree.build(td, **kw)
        torch.cuda.synchronize()
        g = kdgb_lib.Graph(tree, td, params=kdgb_lib.build_params(**kw), headroom=1.5, stream=build_s)
        g.launch(stream=build_s)
        assert g.status(stream=build_s) == 0
        h = tree.to_host()
        for f in ("info", "split", "children", "bitmap", "prim_indices"):
            a, b = getattr(h, f), getattr(ref, f)
            assert np.array_equal(a.view(np.uint32) if a.dtype.kind == "f" else a,
                                  b.view(np.uint32) if b.dtype.kind == "f" else b), f
        trace_s.wait_stream(build_s)
        got = [x.cpu().numpy() for x in tree.trace_primary_shadow(od, dd, (0.5, 3.0, 0.5), tp, stream=trace_s)]
        torch.cuda.synchronize()
        for a, b in zip(got, want):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        g.close()
        tree.close()
