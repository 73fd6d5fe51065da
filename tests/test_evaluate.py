"""World-space evaluation (CompressedShadowContainer::evaluate,
src/CompressedShadowContainer.cpp:93-124 and shader/traverse.cs:134-148):
positions times the light view-projection, perspective divide, grid lookup,
and the percentage-closer filter the reference declares (setFilterSize) but
never applies.  The oracle's restatement is pinned to its own grid lookup on
the CPU; the GPU path must equal it byte for byte."""
import numpy as np
import pytest

from cpvs_gb300 import scene

N, L = 64, 2  # 2x2 xy tiles of 64^2, 2 z-tiles: dag_levels 7, grid_levels 1


def ortho_light():
    """A rotated orthographic light: world box [0,10]^3 -> NDC, column vectors."""
    a = 0.3
    R = np.array([[np.cos(a), -np.sin(a), 0, 0], [np.sin(a), np.cos(a), 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]])
    S = np.diag([0.2, 0.2, 0.2, 1.0])
    T = np.eye(4)
    T[:3, 3] = -1.0
    return (T @ S @ R).astype(np.float32)  # R first, then scale, then shift


def persp_light():
    """A projective matrix with w in about [1, 3] over the position range."""
    M = np.eye(4, dtype=np.float32) * np.float32(0.15)
    M[3, :] = np.array([0.05, 0.03, 0.1, 1.0], np.float32)
    M[:3, 3] = np.float32(-0.9)
    return M


def positions(h, w, fpp, seed):
    g = np.random.default_rng(seed)
    p = g.uniform(-0.5, 10.5, (h, w, fpp)).astype(np.float32)
    p[..., 3:] = np.float32(1.0)
    return p


def grid_inputs(oracle):
    full = scene.rasterise(scene.make_scene(N * L, 0.9, 20, 4, 77))
    tiles, dags, offs, off = {}, [], [], 0
    for z in range(L):
        for y in range(L):
            for x in range(L):
                tile = np.ascontiguousarray(full[y * N:(y + 1) * N, x * N:(x + 1) * N])
                b = oracle.build(tile, z, L)
                tiles[(x, y, z)] = tile
                dags.append(b.dag)
                offs.append(off)
                off += b.dag.size
    return tiles, np.concatenate(dags).astype(np.uint32), np.asarray(offs, np.uint32)


def colmajor(M):
    return np.ascontiguousarray(M.T.ravel(), np.float32)


def test_oracle_evaluate_is_transform_then_grid_lookup(oracle):
    _, dag, offs = grid_inputs(oracle)
    dl = int(np.log2(N)) + 1
    for M in (ortho_light(), persp_light()):
        pos = positions(40, 50, 4, 5)
        m = colmajor(M)
        x, y, z = pos[..., 0].ravel(), pos[..., 1].ravel(), pos[..., 2].ravel()
        c = [((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] for r in range(4)]
        ndc = np.stack([c[0] / c[3], c[1] / c[3], c[2] / c[3]], 1).astype(np.float32)
        want = oracle.grid_lookup_ndc(dag, offs, L, dl, True, ndc)
        got = oracle.grid_evaluate(dag, offs, L, dl, True, pos, m, 1)
        assert np.array_equal(got.ravel(), np.where(want == 1, 255, 0).astype(np.uint8))


def test_oracle_pcf_fraction(oracle):
    _, dag, offs = grid_inputs(oracle)
    dl = int(np.log2(N)) + 1
    pos = positions(30, 30, 3, 6)
    m = colmajor(ortho_light())
    one = oracle.grid_evaluate(dag, offs, L, dl, True, pos, m, 1)
    three = oracle.grid_evaluate(dag, offs, L, dl, True, pos, m, 3)
    # a fully lit or fully shadowed footprint agrees with the centre sample
    assert np.all((three != 255) | (one == 255)) and np.all((three != 0) | (one == 0))
    assert len(np.unique(three)) > 2  # partial footprints exist
    assert set(np.unique(three)) <= {int((255 * k + 4) // 9) for k in range(10)}


@pytest.mark.gpu
def test_evaluate_matches_oracle(cp, oracle):
    tiles, dag, offs = grid_inputs(oracle)
    dl = int(np.log2(N)) + 1
    grid = cp.CompressedShadowContainer(L)
    for (x, y, z), tile in tiles.items():
        grid.set(cp.CompressedShadow.from_depth(tile, z, L), x, y, z)
    grid.copy_to_gpu()
    for M in (ortho_light(), persp_light()):
        for fpp in (3, 4):
            pos = positions(97, 131, fpp, 7 + fpp)
            want = oracle.grid_evaluate(dag, offs, L, dl, True, pos, colmajor(M), 1)
            grid.set_filter_size(1)
            assert np.array_equal(grid.evaluate(pos, M), want)
            bits = grid.evaluate(pos, M, packed=True)
            assert np.array_equal(cp.unpack_bits(bits, pos.shape[0] * pos.shape[1]), (want.ravel() == 255))
            for f in (2, 3, 5):
                grid.set_filter_size(f)
                want_f = oracle.grid_evaluate(dag, offs, L, dl, True, pos, colmajor(M), f)
                assert np.array_equal(grid.evaluate(pos, M), want_f), f
    # device buffers in and out
    import torch
    grid.set_filter_size(3)
    pos = positions(64, 64, 4, 11)
    want = oracle.grid_evaluate(dag, offs, L, dl, True, pos, colmajor(ortho_light()), 3)
    dev = grid.evaluate(torch.from_numpy(pos).cuda(), ortho_light())
    assert np.array_equal(dev.cpu().numpy(), want)
    with pytest.raises(cp.CpvsError):
        grid.evaluate(pos, ortho_light(), packed=True)  # bits need filter size 1


@pytest.mark.gpu
def test_evaluate_single_shadow_container(cp, oracle):
    depth = scene.rasterise(scene.make_scene(256, 0.9, 40, 4, 12))
    b = oracle.build(depth)
    c = cp.CompressedShadowContainer.of(cp.CompressedShadow.from_depth(depth))
    c.copy_to_gpu()
    pos = positions(128, 128, 4, 13)
    M = ortho_light()
    want = oracle.grid_evaluate(b.dag.astype(np.uint32), np.zeros(1, np.uint32), 1, b.num_levels, True, pos,
                                colmajor(M), 1)
    assert np.array_equal(c.evaluate(pos, M), want)
