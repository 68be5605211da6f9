"""Adjoint (kdgb_backward): gradients of first-hit t, u, v with respect to
the vertices of an indexed height-field mesh, reusing the forward's hit ids.

Checked against (a) an FP64 brute-force reference gradient (the same closed
form in double precision over every ray), (b) FP64 central finite
differences with step h = 1e-4 on 256 random vertices, and (c)
torch.autograd.gradcheck through a torch.autograd.Function wrapper (this
harness only).  The central differences use the fourth-order stencil
(8(L(x+h) - L(x-h)) - (L(x+2h) - L(x-2h))) / 12h: with the second-order
stencil the truncation error alone is ~1e-3 relative on this mesh, whose
triangle edges are only 3-6e-3 long.
"""
import numpy as np
import pytest

from kdgb import scenes

pytestmark = pytest.mark.gpu

REL = 1e-4  # relative tolerance of the contract
EPS32 = 2.0 ** -24
# Per-component check: |g - G| <= REL * |G| + FLOOR, where the floor is the
# fp32 rounding that the closed form cannot avoid, summed over the rays that
# make up the component:
#   C_TERM * B  first-order rounding bound of each ray's term (B, below),
#               dominated by the barycentric weights: u = (p . s) / det adds
#               products of size |p||s| that cancel to u * det when the ray
#               origin is far from the small triangle (here 1.5 units from
#               edges of 3e-3), so fp32 u and v carry ~1e-5 relative error;
#   K * EPS32 * A  fp32 accumulation of the K terms of the component
#               (A = sum of their magnitudes).
# Measured against an fp32 restatement of the kernel, each term's error stays
# below 1.2 B, so C_TERM = 4 leaves a margin of more than 3.
C_TERM = 4.0


def mt64(V, idx, hit, o, d):
    """FP64 Moeller-Trumbore for fixed hit triangles."""
    h = np.maximum(hit, 0)
    v0, v1, v2 = V[idx[3 * h]], V[idx[3 * h + 1]], V[idx[3 * h + 2]]
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d, e2)
    s = o - v0
    q = np.cross(s, e1)
    inv = 1.0 / np.einsum("ij,ij->i", p, e1)
    t = inv * np.einsum("ij,ij->i", q, e2)
    u = inv * np.einsum("ij,ij->i", p, s)
    v = inv * np.einsum("ij,ij->i", q, d)
    m = hit >= 0
    return np.where(m, t, 0.0), np.where(m, u, 0.0), np.where(m, v, 0.0)


def rounding_floor(V, idx, hit, o, d, gt, gu, gv):
    """Per component (V.shape): the floor of the per-component check,
    C_TERM * B + K * EPS32 * A (see the module constants), from FP64
    quantities.  B bounds each term w_k * lambda (w = 1 - u - v, u, v) to
    first order: |w_k| d(lambda) + d(w_k) |lambda|, with
      du = eps (sum|p_i s_i| + sum|p_i| (|o_i| + |v0_i|) + |u| sum|p_i e1_i|) / |det|
      dv likewise with q . d (q = s x e1, s itself rounded),
      d(lambda_j) = eps (sum_k |g_k| |vec_k,j|) / |D| + eps |lambda_j| sum|d_i n_i| / |D|,
    where n = e1 x e2, D = d . n and vec = (n, d x e2, d x e1)."""
    m = hit >= 0
    h, o, d, gt, gu, gv = hit[m], o[m], d[m], gt[m], gu[m], gv[m]
    i0, i1, i2 = idx[3 * h], idx[3 * h + 1], idx[3 * h + 2]
    v0, v1, v2 = V[i0], V[i1], V[i2]
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d, e2)
    s = o - v0
    q = np.cross(s, e1)
    det = np.einsum("ij,ij->i", p, e1)
    u = np.einsum("ij,ij->i", p, s) / det
    v = np.einsum("ij,ij->i", q, d) / det
    n = np.cross(e1, e2)
    D = np.einsum("ij,ij->i", d, n)
    de2, de1 = np.cross(d, e2), np.cross(d, e1)
    lam = (gt[:, None] * n + gu[:, None] * de2 - gv[:, None] * de1) / D[:, None]
    ad = np.abs(det)
    pe = (np.abs(p) * np.abs(e1)).sum(1)
    du = EPS32 * ((np.abs(p) * np.abs(s)).sum(1) + (np.abs(p) * (np.abs(o) + np.abs(v0))).sum(1) + np.abs(u) * pe) / ad
    s_mag = np.abs(s) + np.abs(o) + np.abs(v0)
    dv = EPS32 * ((np.abs(np.cross(s_mag, np.abs(e1))) * np.abs(d)).sum(1) + (np.abs(q) * np.abs(d)).sum(1) +
                  np.abs(v) * pe) / ad
    dlam = EPS32 * (np.abs(gt)[:, None] * np.abs(n) + np.abs(gu)[:, None] * np.abs(de2) +
                    np.abs(gv)[:, None] * np.abs(de1)) / np.abs(D)[:, None] + \
        EPS32 * np.abs(lam) * ((np.abs(d) * np.abs(n)).sum(1) / np.abs(D))[:, None]
    w0 = 1 - u - v
    B = np.zeros_like(V)
    A = np.zeros_like(V)
    K = np.zeros(V.shape[0])
    for ii, wk, dwk in ((i0, w0, du + dv), (i1, u, du), (i2, v, dv)):
        np.add.at(B, ii, np.abs(wk)[:, None] * dlam + dwk[:, None] * np.abs(lam))
        np.add.at(A, ii, np.abs(wk[:, None] * lam))
        np.add.at(K, ii, 1.0)
    return C_TERM * B + K[:, None] * EPS32 * A


def grad64(V, idx, hit, o, d, gt, gu, gv):
    """FP64 brute-force reference gradient: closed form over every ray."""
    m = hit >= 0
    h, o, d, gt, gu, gv = hit[m], o[m], d[m], gt[m], gu[m], gv[m]
    i0, i1, i2 = idx[3 * h], idx[3 * h + 1], idx[3 * h + 2]
    v0, v1, v2 = V[i0], V[i1], V[i2]
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d, e2)
    s = o - v0
    q = np.cross(s, e1)
    inv = 1.0 / np.einsum("ij,ij->i", p, e1)
    u = inv * np.einsum("ij,ij->i", p, s)
    v = inv * np.einsum("ij,ij->i", q, d)
    n = np.cross(e1, e2)
    lam = (gt[:, None] * n + gu[:, None] * np.cross(d, e2) - gv[:, None] * np.cross(d, e1)) / \
        np.einsum("ij,ij->i", d, n)[:, None]
    G = np.zeros_like(V)
    np.add.at(G, i0, (1 - u - v)[:, None] * lam)
    np.add.at(G, i1, u[:, None] * lam)
    np.add.at(G, i2, v[:, None] * lam)
    return G


@pytest.fixture(scope="module")
def c5(kdgb_lib, cuda):
    """316x158 height field (99,856 triangles, 50,403 vertices), 512x512
    primary rays, loss sum_r w_r t_r + a_r (u_r + v_r), w, a ~ N(0,1)."""
    nx, ny = 316, 158
    verts = scenes.heightfield_vertices(nx, ny, seed=1)
    idx = scenes.grid_indices(nx, ny)
    tris = verts[idx.astype(np.int64)].reshape(-1, 9)
    o, d = scenes.camera_rays(512, 512)
    with kdgb_lib.KDTree.build(tris) as tree:
        hit, t, u, v = (x.cpu().numpy() for x in tree.trace(o, d, tracer=kdgb_lib.TRACER_RESTART))
    w = scenes.normal(5, o.shape[0], 0).astype(np.float32)
    a = scenes.normal(5, o.shape[0], 1).astype(np.float32)
    g = kdgb_lib.backward(verts, idx, o, d, hit, w, a, a).cpu().numpy()
    return dict(verts=verts, idx=idx.astype(np.int64), o=o, d=d, hit=hit, t=t, u=u, v=v, w=w, a=a, g=g)


def test_forward_shape(c5):
    assert c5["verts"].shape == (50403, 3) and c5["idx"].shape == (99856 * 3,)
    assert (c5["hit"] >= 0).mean() > 0.3


def _fp64_args(c5):
    return (c5["idx"], c5["hit"], c5["o"].astype(np.float64), c5["d"].astype(np.float64),
            c5["w"].astype(np.float64), c5["a"].astype(np.float64), c5["a"].astype(np.float64))


def test_against_fp64_reference_gradient(c5):
    V = c5["verts"].astype(np.float64)
    G = grad64(V, *_fp64_args(c5))
    floor = rounding_floor(V, *_fp64_args(c5))
    g = c5["g"].astype(np.float64)
    rel = np.linalg.norm(g - G) / np.linalg.norm(G)
    assert rel < REL, rel
    # Component by component, over all 151,209 components.
    err = np.abs(g - G)
    bound = REL * np.abs(G) + floor
    bad = err > bound
    assert not bad.any(), (int(bad.sum()), float((err[bad] / bound[bad]).max()))
    # The contract's 1e-4 alone holds for most components (an fp32
    # restatement of the kernel meets it on 92% of the touched ones; the
    # median relative error is 1e-5).
    touched = np.abs(G) > 0
    assert (err <= REL * np.abs(G))[touched].mean() > 0.85
    touched = np.abs(G).sum(1) > 0
    assert (np.abs(g[~touched]) == 0).all()


def test_against_fp64_central_differences(c5):
    V = c5["verts"].astype(np.float64)
    idx, hit = c5["idx"], c5["hit"]
    o, d = c5["o"].astype(np.float64), c5["d"].astype(np.float64)
    w, a = c5["w"].astype(np.float64), c5["a"].astype(np.float64)
    g = c5["g"].astype(np.float64)
    cand = np.nonzero(np.abs(g).sum(1) > 0)[0]
    sel_v = cand[(scenes.uniform(6, 256, 0) * len(cand)).astype(np.int64)]
    h = 1e-4
    tri_vid = idx.reshape(-1, 3)
    floor = rounding_floor(V, *_fp64_args(c5))
    num, ana, mag = [], [], []
    for j in sel_v:
        rays = np.nonzero(np.isin(hit, np.nonzero((tri_vid == j).any(1))[0]))[0]
        for c in range(3):
            L = {}
            for k in (-2, -1, 1, 2):
                Vp = V.copy()
                Vp[j, c] += k * h
                tt, uu, vv = mt64(Vp, idx, hit[rays], o[rays], d[rays])
                L[k] = np.sum(w[rays] * tt + a[rays] * (uu + vv))
            num.append((8 * (L[1] - L[-1]) - (L[2] - L[-2])) / (12 * h))
            ana.append(g[j, c])
            mag.append(floor[j, c])
    num, ana, mag = np.array(num), np.array(ana), np.array(mag)
    rel = np.linalg.norm(ana - num) / np.linalg.norm(num)
    assert rel < REL, rel
    # Each of the 768 sampled components on its own.
    err = np.abs(ana - num)
    bound = REL * np.abs(num) + mag
    assert (err <= bound).all(), (int((err > bound).sum()), float((err / bound).max()))


def test_backward_accumulates_and_ignores_misses(kdgb_lib, cuda, c5):
    import torch
    g1 = kdgb_lib.backward(c5["verts"], c5["idx"].astype(np.uint32), c5["o"], c5["d"], c5["hit"], c5["w"], c5["a"],
                           c5["a"])
    g2 = kdgb_lib.backward(c5["verts"], c5["idx"].astype(np.uint32), c5["o"], c5["d"], c5["hit"], c5["w"], c5["a"],
                           c5["a"], out=g1.clone())
    # Float atomics: the summation order differs between calls, so compare in
    # norm (vertices whose contributions cancel have large relative noise).
    assert float((g2 - 2 * g1).norm() / (2 * g1).norm()) < 1e-6
    none = np.full_like(c5["hit"], -1)
    g0 = kdgb_lib.backward(c5["verts"], c5["idx"].astype(np.uint32), c5["o"], c5["d"], none, c5["w"], c5["a"],
                           c5["a"])
    assert float(g0.abs().sum()) == 0.0


def test_gradcheck_through_autograd_function(kdgb_lib, cuda):
    """torch.autograd.gradcheck of t, u, v w.r.t. the vertices of a coarse
    mesh; the forward builds and traces on the GPU, the backward is
    kdgb_backward."""
    import torch

    verts0 = scenes.heightfield_vertices(6, 6, seed=3)
    idx = scenes.grid_indices(6, 6)
    idx_t = torch.from_numpy(idx.astype(np.int32)).cuda()
    # Rays through triangle interiors (away from edges) so that the small
    # perturbations of gradcheck never move a hit to another triangle.
    tris0 = verts0[idx.astype(np.int64)].reshape(-1, 3, 3)
    pick = np.arange(0, tris0.shape[0], 5)
    centers = tris0[pick].mean(1)
    o = np.ascontiguousarray(centers + np.array([0.013, -0.007, 1.0], np.float32), np.float32)
    d = np.tile(np.array([0.0, 0.0, -1.0], np.float32), (o.shape[0], 1))
    o_t, d_t = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()

    def trace(V):
        tris = V.detach()[idx_t.long()].reshape(-1, 9).contiguous()
        with kdgb_lib.KDTree.build(tris) as tree:
            return tree.trace(o_t, d_t, tracer=kdgb_lib.TRACER_RESTART)

    hit0 = trace(torch.from_numpy(verts0).cuda())[0]
    assert (hit0 >= 0).all()

    class KdTrace(torch.autograd.Function):
        @staticmethod
        def forward(ctx, V):
            hit, t, u, v = trace(V)
            assert torch.equal(hit, hit0), "a perturbation moved a hit"
            ctx.save_for_backward(V)
            return t, u, v

        @staticmethod
        def backward(ctx, gt, gu, gv):
            (V,) = ctx.saved_tensors
            return kdgb_lib.backward(V.detach(), idx_t, o_t, d_t, hit0, gt.contiguous(), gu.contiguous(),
                                     gv.contiguous())

    V = torch.from_numpy(verts0).cuda().requires_grad_(True)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert torch.autograd.gradcheck(KdTrace.apply, (V,), eps=1e-3, atol=5e-3, rtol=5e-3, nondet_tol=1e-5)
