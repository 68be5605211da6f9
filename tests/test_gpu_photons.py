"""Photon workload (incoherent rays): kdgb_trace_photons against the oracle's
restatement on the same tree, and the Philox4x32-10 block against cuRAND's."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
LIGHT = (0.5, 0.5, 0.5)


@pytest.fixture(scope="module")
def photon_scene(oracle):
    tris = scenes.clustered(60000, seed=2)
    return tris, oracle.build(tris, **SAH_C1)


@pytest.mark.parametrize("tracer", [0, 1])
def test_photons_match_oracle(kdgb_lib, cuda, oracle, photon_scene, tracer):
    tris, tree = photon_scene
    n = 40000
    ref_h, ref_t = oracle.trace_photons(tree, tris, n, light=LIGHT, seed=11, tracer=tracer, stack_depth=8)
    ph = kdgb_lib.photon_params(light=LIGHT, seed=11)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        h, t = gt.trace_photons(n, photons=ph, tracer=tracer, stack_depth=8)
        h, t = h.cpu().numpy(), t.cpu().numpy()
    assert np.array_equal(h, ref_h), f"{(h != ref_h).sum()} segment ids differ"
    m = ref_h >= 0
    assert np.array_equal(t[m].view(np.uint32), ref_t[m].view(np.uint32))
    # Every bounce level is exercised.
    assert all((ref_h[:, k] >= 0).sum() > 20 for k in range(4))
    # Segments after the end of a photon are marked -2, never followed by a hit.
    ended = np.cumsum(ref_h < 0, axis=1) > 0
    assert (ref_h[:, 1:][ended[:, :-1]] == -2).all()


def test_photons_restart_equals_shortstack(kdgb_lib, cuda, photon_scene):
    tris, tree = photon_scene
    ph = kdgb_lib.photon_params(light=LIGHT, seed=5)
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        a = gt.trace_photons(20000, photons=ph, tracer=0)[0].cpu().numpy()
        b = gt.trace_photons(20000, photons=ph, tracer=1, stack_depth=8)[0].cpu().numpy()
    assert (a == b).mean() > 0.999


def test_photons_on_gpu_built_tree(kdgb_lib, cuda, oracle, photon_scene):
    tris, tree = photon_scene
    ph = kdgb_lib.photon_params(light=LIGHT, seed=7, bounces=2, survival=0.5)
    ref_h, _ = oracle.trace_photons(tree, tris, 10000, light=LIGHT, seed=7, bounces=2, survival=0.5, tracer=1)
    with kdgb_lib.KDTree.build(tris, **SAH_C1) as gt:
        h = gt.trace_photons(10000, photons=ph, tracer=1)[0].cpu().numpy()
    assert h.shape == (10000, 3) and np.array_equal(h, ref_h)


def test_photon_params_validated(kdgb_lib, cuda, photon_scene):
    tris, tree = photon_scene
    with kdgb_lib.KDTree.upload(tree, tris) as gt:
        for bad in (dict(survival=1.5), dict(bounces=-1)):
            with pytest.raises(kdgb_lib.KdgbError) as e:
                gt.trace_photons(16, photons=kdgb_lib.photon_params(**bad))
            assert e.value.status == 1
        with pytest.raises(kdgb_lib.KdgbError) as e:
            gt.trace_photons(16, tracer=2)
        assert e.value.status == 8


def test_philox_matches_curand(kdgb_lib, cuda, tmp_path):
    src = os.path.join(HERE, "helpers", "philox_curand.cu")
    lib = str(tmp_path / "libphilox_test.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--fmad=false",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "extensions-photonmapping_gb300",
                                                                            "csrc"),
                    "-Xcompiler", "-fPIC", "-shared", src, "-o", lib], check=True)
    L = C.CDLL(lib)
    n = 4096
    ours = np.zeros((n, 4), np.uint32)
    theirs = np.zeros((n, 4), np.uint32)
    assert L.philox_compare(ours.ctypes.data_as(C.c_void_p), theirs.ctypes.data_as(C.c_void_p), n) == 0
    assert np.array_equal(ours, theirs)


def test_oracle_philox_matches_device(kdgb_lib, cuda, oracle, tmp_path):
    # The oracle's Philox (host C) gives the same block as the device one
    # on the counters the helper uses.
    i = 123
    ctr = [(2654435761 * i) & 0xffffffff, i, i ^ 0xdeadbeef, 7]
    key = [0x12345678 + i, 0x9abcdef0]
    out = oracle.philox4x32_10(ctr, key)
    src = os.path.join(HERE, "helpers", "philox_curand.cu")
    lib = str(tmp_path / "libphilox_test2.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--fmad=false",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "extensions-photonmapping_gb300",
                                                                            "csrc"),
                    "-Xcompiler", "-fPIC", "-shared", src, "-o", lib], check=True)
    L = C.CDLL(lib)
    ours = np.zeros((i + 1, 4), np.uint32)
    theirs = np.zeros((i + 1, 4), np.uint32)
    assert L.philox_compare(ours.ctypes.data_as(C.c_void_p), theirs.ctypes.data_as(C.c_void_p), i + 1) == 0
    assert np.array_equal(ours[i], out)
