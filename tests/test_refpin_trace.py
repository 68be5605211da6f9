"""The oracle's tracers and shading loop, checked bit for bit against the
reference's OWN tracer sources.

`oracle/refpin/Makefile` compiles Utils/CUDA/Raytracer.cu, ShortStack.cu and
BruteTracer.cu unmodified with nvcc (`-cudart none`). The stand-ins of
`oracle/refpin/include_cu` cover OpenEngine core, cutil and the CUDA SDK
helpers. `oracle/refpin/refpin_runtime.cpp` answers the CUDA runtime calls
of the fetch helpers' host branch with host copies. The reference's
`__host__ __device__` traversal functions then run on the CPU, ray by ray, as
its HostTrace methods call them:
- KDRestart and ShadowRay (kd-restart);
- ShortStackTrace (short stack);
- Exhaustive (brute force).

The reference's own debug log lines (CUDALogger "THit:" and "Primary ray
intersected") report each ray's hits.

The one substitution: the specular power of ColorKernels.h. Its device path
calls __powf and its host path the C library's powf. The pin installs the
oracle's own or_kpow, which the CUDA kernel computes too. A separate test
bounds what the C library's powf changes.

The library is built into oracle/_ref where the reference tree and nvcc are
available. Elsewhere these tests skip.
"""
import numpy as np
import pytest

from kdgb import scenes


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.refpin_trace_lib() is None:
        pytest.skip("the reference tree (or nvcc) is not available to compile the tracer pin library")
    return oracle


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


SAH_C1 = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)


@pytest.mark.parametrize("tree_kw", [dict(), SAH_C1], ids=["bitmap", "sah"])
@pytest.mark.parametrize("intersection", [0, 1], ids=["moeller", "woop"])
@pytest.mark.parametrize("tracer,leaf_skipping", [(0, True), (0, False), (1, True), (1, False), (2, True)],
                         ids=["restart", "restart-noskip", "shortstack", "shortstack-noskip", "brute"])
def test_shaded_pixels_pinned(ref, tree_kw, intersection, tracer, leaf_skipping):
    """Whole shading loop: traversal, hit, Phong light, reflection and
    blending until alpha 0.97 (Raytracer.cu:165-262, ShortStack.cu:96-194,
    BruteTracer.cu:54-96, ColorKernels.h:15-85)."""
    tris, n0, n1, n2, c0 = scenes.shaded_box(32, 16, seed=3)
    o, d = scenes.camera_rays(96, 64)
    tree = ref.build(tris, **tree_kw)
    got, _ = ref.ref_trace(tracer, tree, tris, o, d, n0, n1, n2, c0, intersection=intersection,
                           leaf_skipping=leaf_skipping)
    want = ref.trace_shaded(tree if tracer != 2 else None, tris, o, d, n0, n1, n2, c0, tracer=tracer,
                            stack_depth=4, intersection=intersection, leaf_skipping=int(leaf_skipping),
                            max_bounces=1 << 20)
    assert np.array_equal(got, want), int((got != want).any(axis=1).sum())
    assert (want[:, 3] > 0).mean() > 0.5
    assert len(np.unique(want[:, 3])) > 3  # multi-bounce pixels


def test_shaded_pixels_other_light(ref):
    tris, n0, n1, n2, c0 = scenes.shaded_box(16, 8, seed=4)
    o, d = scenes.camera_rays(64, 32)
    L = dict(position=(0.5, 0.5, 3.0), ambient=(0.1, 0.1, 0.1), diffuse=(0.8, 0.7, 0.6), specular=(0.5, 0.5, 0.5))
    tree = ref.build(tris)
    for tracer in (0, 1):
        got, _ = ref.ref_trace(tracer, tree, tris, o, d, n0, n1, n2, c0, light_params=ref.light(**L))
        want = ref.trace_shaded(tree, tris, o, d, n0, n1, n2, c0, light_params=ref.light(**L), tracer=tracer,
                                stack_depth=4, max_bounces=1 << 20)
        assert np.array_equal(got, want)
        default, _ = ref.ref_trace(tracer, tree, tris, o, d, n0, n1, n2, c0)
        assert (default != got).any(axis=1).mean() > 0.2  # the light reaches the pixels


def test_library_powf_changes_little(ref):
    """With the C library's powf (the reference's real host path) instead of
    or_kpow, no channel moves by more than 1 and few pixels move at all."""
    tris, n0, n1, n2, c0 = scenes.shaded_box(32, 16, seed=5)
    o, d = scenes.camera_rays(96, 64)
    tree = ref.build(tris)
    a, _ = ref.ref_trace(0, tree, tris, o, d, n0, n1, n2, c0)
    b, _ = ref.ref_trace(0, tree, tris, o, d, n0, n1, n2, c0, oracle_pow=False)
    diff = np.abs(a.astype(np.int32) - b.astype(np.int32))
    assert diff.max() <= 1
    assert (diff > 0).any(axis=1).mean() < 0.01


def _scene(name):
    if name == "clustered":
        return scenes.clustered(6000, seed=4)
    if name == "heightfield":
        return scenes.heightfield(64, 32, seed=1)[0]
    rng = np.random.default_rng(7)
    c = rng.random((3000, 1, 3)).astype(np.float32)
    tris = (c + rng.normal(size=(3000, 3, 3)).astype(np.float32) * 0.05).reshape(-1, 9)
    tris[::9, 3:6] = tris[::9, 0:3]  # degenerate triangles
    return tris


def _rays(tris, n, seed):
    rng = np.random.default_rng(seed)
    p = tris.reshape(-1, 3)
    lo, hi = p.min(0), p.max(0)
    o = (lo + (hi - lo) * rng.uniform(-0.2, 1.2, size=(n, 3))).astype(np.float32)
    tgt = tris.reshape(-1, 3, 3)[rng.integers(0, tris.shape[0], n)].mean(1)
    d = (tgt - o).astype(np.float32)
    d[::3] = rng.normal(size=(len(d[::3]), 3)).astype(np.float32)  # some rays miss
    d[::17, 1] = 0.0                                                # axis-parallel components
    return o, d


TREES = {"bitmap": dict(), "sah": dict(lower=1), "balanced": dict(lower=2), "divide": dict(split_method=1),
         "sah_c1": SAH_C1}


@pytest.mark.parametrize("tree", list(TREES))
@pytest.mark.parametrize("scene", ["clustered", "heightfield", "soup"])
def test_first_hits_pinned(ref, tree, scene):
    """First hits, from the reference's own log lines: kd-restart's primitive
    and tHit (t, u, v) (Raytracer.cu:226-230), and the short stack's tHit
    after its last leaf with opaque colours, which end the loop at the first
    hit (ShortStack.cu:169).  Both intersection methods."""
    tris = _scene(scene)
    t_kw = TREES[tree]
    tr = ref.build(tris, **t_kw)
    o, d = _rays(tris, 8000, seed=11)
    nn = np.tile(np.array([0, 1, 0, 0], np.float32), (tris.shape[0], 1))
    opaque = np.full((tris.shape[0], 4), 255, np.uint8)
    for isect in (0, 1):
        _, (prim, th) = ref.ref_trace(0, tr, tris, o, d, nn, nn, nn, opaque, intersection=isect)
        hit, t, u, v = ref.trace(tr, tris, o, d, intersection=isect)
        m = hit >= 0
        assert np.array_equal(prim, hit)
        for k, x in enumerate((t, u, v)):
            assert np.array_equal(bits(th[m, k]), bits(x[m])), (isect, k)
        assert 0.3 < m.mean() < 1.0

        rgba, last = ref.ref_trace(1, tr, tris, o, d, nn, nn, nn, opaque, intersection=isect)
        hit, t, u, v = ref.trace(tr, tris, o, d, intersection=isect, tracer=1, stack_depth=4)
        m = hit >= 0
        assert np.array_equal(rgba[:, 3] > 0, m)
        for k, x in enumerate((t, u, v)):
            assert np.array_equal(bits(last[m, k]), bits(x[m])), (isect, k)


@pytest.mark.parametrize("tree", ["bitmap", "sah", "divide"])
def test_shadow_rays_pinned(ref, tree):
    """ShadowRay (Raytracer.cu:108-163): from the light to each point."""
    tris = _scene("heightfield")
    tr = ref.build(tris, **TREES[tree])
    rng = np.random.default_rng(13)
    p = tris.reshape(-1, 3)
    lo, hi = p.min(0), p.max(0)
    pts = (lo + (hi - lo) * rng.uniform(0, 1, size=(20000, 3))).astype(np.float32)
    light = ((lo + hi) * 0.5).astype(np.float32)
    light[1] = hi[1] + (hi[1] - lo[1])  # above the height field: points under it are in shadow
    for isect in (0, 1):
        lit = ref.ref_shadow(tr, tris, pts, light, intersection=isect)
        occ = ref.trace_shadow(tr, tris, pts, light, intersection=isect)
        assert np.array_equal(lit == 0.0, occ == 1)
        assert 0.05 < occ.mean() < 0.95


def test_brute_cap(ref):
    """Exhaustive tests only the first MAX_PRIMS triangles (BruteTracer.cu:50,
    62); the oracle lifts the cap, so the two agree up to that size."""
    assert ref.refpin_trace_lib().ref_brute_max_prims() == 4096
    assert ref.refpin_trace_lib().ref_shortstack_depth() == 4
