"""Triangle depth rasterisation (cpvs_raster_triangles): the GPU map equals
the host rasteriser (cpvs_gb300/scene.py) bit for bit -- random triangles of
both windings and every size, degenerate and NaN ones, a seamless terrain
mesh, windows, device buffers -- and a DAG built from a rasterised mesh
equals the oracle's."""
import numpy as np
import pytest

from cpvs_gb300 import scene


def same_map(a, b):
    """Bit-identical, except that NaNs compare by position only (arithmetic
    NaNs carry an implementation-defined payload; every comparison against
    any NaN is false, so the DAG does not depend on it)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def random_tris(rng, m):
    t = rng.uniform(-0.1, 1.1, (m, 9)).astype(np.float32)
    t[:, 2::3] = rng.uniform(0.1, 0.95, (m, 3)).astype(np.float32)
    small = rng.random(m) < 0.5  # half of them small: a vertex plus short offsets
    for k in (3, 6):
        t[small, k] = t[small, 0] + rng.uniform(-0.02, 0.02, small.sum()).astype(np.float32)
        t[small, k + 1] = t[small, 1] + rng.uniform(-0.02, 0.02, small.sum()).astype(np.float32)
    t[0, 3:5] = t[0, 0:2]          # degenerate: two equal vertices
    t[1, 6:8] = (t[1, 0:2] + t[1, 3:5]) / 2  # degenerate-ish: collinear midpoint
    t[2, 5] = np.float32(np.nan)    # NaN depth propagates
    t[3, 0] = np.float32(np.nan)    # NaN position: skipped
    return t


def test_host_terrain_is_seamless():
    n = 64
    t = scene.terrain_triangles(8, 3)
    d = scene.rasterise_triangles(t, n, 1.0)
    assert (d < 1.0).all()  # every pixel centre lies in some triangle of the mesh
    assert d.min() >= 0.3 - 1e-6 and d.max() <= 0.8 + 1e-6


def test_host_right_triangle_coverage():
    n = 16
    t = np.array([[0, 0, 0.5, 1, 0, 0.5, 0, 1, 0.5]], np.float32)  # lower-left half, constant depth
    d = scene.rasterise_triangles(t, n, 1.0)
    c = scene.pixel_centres(n)
    want = (c[None, :] + c[:, None]) <= 1.0
    assert np.array_equal(d == np.float32(0.5), want)


@pytest.mark.gpu
def test_triangles_match_host(cp):
    rng = np.random.default_rng(4)
    for n, m in ((64, 50), (256, 400), (1024, 3000)):
        t = random_tris(rng, m)
        want = scene.rasterise_triangles(t, n, 0.97)
        got = cp.raster_triangles(t, n, 0.97)
        assert same_map(got, want), n


@pytest.mark.gpu
def test_terrain_windows_and_device_io(cp):
    import torch
    n = 512
    t = scene.terrain_triangles(24, 9)
    full = scene.rasterise_triangles(t, n, 1.0)
    assert np.array_equal(cp.raster_triangles(t, n, 1.0).view(np.uint32), full.view(np.uint32))
    win = cp.raster_triangles(t, n, 1.0, x0=96, y0=200, w=130, h=70)
    assert np.array_equal(win.view(np.uint32), full[200:270, 96:226].view(np.uint32))
    dev = cp.raster_triangles(torch.from_numpy(t).cuda(), n, 1.0)
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), full.view(np.uint32))
    assert cp.raster_triangles(np.zeros((0, 9), np.float32), 64, 0.5).min() == np.float32(0.5)


@pytest.mark.gpu
def test_dag_of_a_rasterised_mesh_matches_oracle(cp, oracle):
    n = 1024
    t = np.concatenate([scene.terrain_triangles(16, 5, 0.5, 0.9), random_tris(np.random.default_rng(6), 200)[4:]])
    depth = cp.raster_triangles(t, n, 0.95)
    assert np.array_equal(depth.view(np.uint32), scene.rasterise_triangles(t, n, 0.95).view(np.uint32))
    sh = cp.CompressedShadow.from_depth(depth)
    assert np.array_equal(sh.get_dag(), oracle.build(depth).dag)
