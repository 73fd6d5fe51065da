"""The deferred shading pass (shader/shade.frag:34-56) on G-buffer images.

Every float operation of the shader is restated as one IEEE round-to-nearest
float32 step in a fixed order, so the oracle (C++, no contraction), a numpy
float32 restatement and the GPU kernel agree bit for bit: the tolerance is
zero.  Both branches of the shader are covered: the precomputed visibilities
of evaluate (renderShadow != 0) and the plain shadow-map test
(renderShadow == 0), including texels outside the map (border depth 1.0)."""
import numpy as np
import pytest

from cpvs_gb300 import scene

f32 = np.float32


def gbuffer(h, w, fpn, seed):
    g = np.random.default_rng(seed)
    nrm = g.normal(size=(h, w, fpn)).astype(f32)
    nrm[..., :3] /= np.linalg.norm(nrm[..., :3], axis=-1, keepdims=True).astype(f32)
    alb = g.uniform(0, 1, (h, w, 4)).astype(f32)
    vis = g.choice(np.array([0, 255, 17, 128], np.uint8), size=(h, w), p=[0.4, 0.4, 0.1, 0.1])
    pos = g.uniform(-1.0, 11.0, (h, w, 4)).astype(f32)  # partly outside the light's box
    pos[..., 3] = f32(1.0)
    return nrm, alb, vis, pos


def ortho_light():
    """World box [0,10]^3 -> clip space, slightly rotated, w = 1."""
    a = 0.2
    R = np.array([[np.cos(a), -np.sin(a), 0, 0], [np.sin(a), np.cos(a), 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]])
    S = np.diag([0.2, 0.2, 0.2, 1.0])
    T = np.eye(4)
    T[:3, 3] = -1.0
    return (T @ S @ R).astype(f32)


def persp_light():
    M = np.eye(4, dtype=f32) * f32(0.15)
    M[3, :] = np.array([0.05, 0.03, 0.1, 1.0], f32)
    M[:3, 3] = f32(-0.9)
    return M


def colmajor(M):
    return np.ascontiguousarray(M.T.ravel(), f32)


def numpy_shade(nrm, alb, light, vis=None, pos=None, sm=None, m=None):
    """The same arithmetic in numpy float32 (elementwise, no contraction)."""
    light = np.asarray(light, f32)
    ln = np.sqrt(light[0] * light[0] + light[1] * light[1] + light[2] * light[2])
    L = light / ln
    if vis is not None:
        v = vis.astype(f32) / f32(255.0)
        v = np.maximum(v, f32(0))
    else:
        x, y, z = pos[..., 0], pos[..., 1], pos[..., 2]
        c = [((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] for r in range(4)]
        s = [(c[k] / c[3]) * f32(0.5) + f32(0.5) for k in range(3)]
        side = f32(sm.shape[0])
        fx, fy = np.floor(s[0] * side), np.floor(s[1] * side)
        inside = (fx >= 0) & (fx < side) & (fy >= 0) & (fy < side)
        ix = np.where(inside, fx, 0).astype(np.int64)
        iy = np.where(inside, fy, 0).astype(np.int64)
        d = np.where(inside, sm[iy, ix], f32(1.0))
        v = np.where(d < s[2], f32(0), f32(1))
    dot = (nrm[..., 0] * L[0] + nrm[..., 1] * L[1]) + nrm[..., 2] * L[2]
    diffuse = np.where(dot > 0, dot, f32(0))
    sc = f32(0.15) + diffuse * v
    out = np.empty(alb.shape, f32)
    out[..., :3] = sc[..., None] * alb[..., :3]
    out[..., 3] = alb[..., 3]
    return out


def test_oracle_shade_with_visibilities_matches_numpy(oracle):
    for fpn in (3, 4):
        nrm, alb, vis, _ = gbuffer(33, 47, fpn, fpn)
        light = (0.3, -1.0, 0.6)
        want = numpy_shade(nrm, alb, light, vis=vis)
        got = oracle.shade(nrm, alb, light, visibilities=vis)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        # lit pixels facing away from the light keep only the ambient term
        back = (nrm[..., :3] @ np.asarray(light, f32)) < 0
        assert np.array_equal(got[back][:, :3], (f32(0.15) * alb[back][:, :3]))


def test_oracle_shadow_map_branch_matches_numpy(oracle):
    depth = scene.rasterise(scene.make_scene(128, 0.9, 30, 4, 5))
    for M in (ortho_light(), persp_light()):
        nrm, alb, _, pos = gbuffer(29, 31, 4, 9)
        m = colmajor(M)
        want = numpy_shade(nrm, alb, (0.1, 0.2, -1.0), pos=pos, sm=depth, m=m)
        got = oracle.shade(nrm, alb, (0.1, 0.2, -1.0), positions=pos, shadow_map=depth, light_view_proj_colmajor=m)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_oracle_shadow_map_border_is_lit(oracle):
    """Positions that project outside the map read the border depth 1.0."""
    depth = np.zeros((16, 16), f32)  # everything in the map is occluded
    nrm = np.zeros((1, 4, 3), f32)
    nrm[..., 2] = 1.0
    alb = np.ones((1, 4, 4), f32)
    M = np.eye(4, dtype=f32)
    pos = np.array([[[0.0, 0.0, 0.5], [2.0, 0.0, 0.5], [0.0, -1.5, 0.5], [0.0, 0.0, 1.5]]], f32)
    got = oracle.shade(nrm, alb, (0, 0, 1), positions=pos, shadow_map=depth, light_view_proj_colmajor=colmajor(M))
    # inside the map: 0 < s.z, shadowed; outside in x or y: 1.0 >= s.z, lit;
    # inside but beyond the far plane (s.z = 1.25): shadowed
    assert got[0, :, 0].tolist() == [np.float32(0.15), np.float32(1.15), np.float32(1.15), np.float32(0.15)]


def test_shade_rejects_bad_arguments_without_a_gpu():
    from cpvs_gb300 import build
    build.build()
    import cpvs_gb300
    lib = cpvs_gb300.load_library()
    light = np.array([0, 0, 1], f32)
    # a null context and a null light are refused before any device call
    assert lib.cpvs_shade(None, 4, 4, None, 3, None, None, None, 0, None, 0, None, light.ctypes.data, None,
                          None) == 1
    assert lib.cpvs_shade(None, 4, 4, None, 3, None, None, None, 0, None, 0, None, None, None, None) == 1


@pytest.mark.gpu
def test_shade_matches_oracle(cp, oracle):
    import torch
    for h, w, fpn in ((1, 1, 4), (97, 131, 4), (64, 65, 3), (200, 8, 4)):
        nrm, alb, vis, pos = gbuffer(h, w, fpn, h + w)
        light = (0.4, 0.7, -0.2)
        want = oracle.shade(nrm, alb, light, visibilities=vis)
        got = cp.shade(nrm, alb, light, visibilities=vis)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (h, w, fpn)
        # device tensors, and a position layout of 4 floats (vector path)
        dn, da, dv = (torch.from_numpy(a).cuda() for a in (nrm, alb, vis))
        got_d = cp.shade(dn, da, light, visibilities=dv)
        assert got_d.is_cuda and np.array_equal(got_d.cpu().numpy().view(np.uint32), want.view(np.uint32))
    # buffers that start off a 16-byte boundary take the scalar path
    nrm, alb, vis, _ = gbuffer(40, 40, 4, 3)
    big = torch.zeros(40 * 40 * 4 + 1, dtype=torch.float32, device="cuda")
    big[1:] = torch.from_numpy(nrm).cuda().reshape(-1)
    dn = big[1:].view(40, 40, 4)
    got = cp.shade(dn, torch.from_numpy(alb).cuda(), (1, 1, 1), visibilities=torch.from_numpy(vis).cuda())
    want = oracle.shade(nrm, alb, (1, 1, 1), visibilities=vis)
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_shade_shadow_map_branch_matches_oracle(cp, oracle):
    depth = scene.rasterise(scene.make_scene(256, 0.9, 40, 4, 21))
    for M in (ortho_light(), persp_light()):
        for fpp in (3, 4):
            nrm, alb, _, pos = gbuffer(73, 91, 4, fpp)
            pos = np.ascontiguousarray(pos[..., :fpp])
            want = oracle.shade(nrm, alb, (0.2, -0.3, -1.0), positions=pos, shadow_map=depth,
                                light_view_proj_colmajor=colmajor(M))
            got = cp.shade(nrm, alb, (0.2, -0.3, -1.0), positions=pos, shadow_map=depth, light_view_proj=M)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (fpp,)
    with pytest.raises(cp.CpvsError):
        cp.shade(nrm, alb, (0, 0, 0), positions=pos, shadow_map=depth, light_view_proj=M)


@pytest.mark.gpu
def test_frame_evaluate_then_shade_matches_oracle(cp, oracle):
    """One frame of the reference's renderer (doAllShading): evaluate the
    precomputed shadow at every G-buffer position, then shade."""
    import torch
    depth = scene.rasterise(scene.make_scene(256, 0.9, 40, 4, 12))
    b = oracle.build(depth)
    c = cp.CompressedShadowContainer.of(cp.CompressedShadow.from_depth(depth))
    c.copy_to_gpu()
    c.set_filter_size(3)
    nrm, alb, _, pos = gbuffer(120, 160, 4, 2)
    M = ortho_light()
    vis_want = oracle.grid_evaluate(b.dag.astype(np.uint32), np.zeros(1, np.uint32), 1, b.num_levels, True, pos,
                                    colmajor(M), 3)
    want = oracle.shade(nrm, alb, (0.3, 0.3, -1.0), visibilities=vis_want)
    dpos = torch.from_numpy(pos).cuda()
    vis = c.evaluate(dpos, M)
    got = cp.shade(torch.from_numpy(nrm).cuda(), torch.from_numpy(alb).cuda(), (0.3, 0.3, -1.0), visibilities=vis)
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32))
