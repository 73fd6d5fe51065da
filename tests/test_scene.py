"""Host-side input synthesis: the seeded scene generator and query sets."""
import numpy as np

from cpvs_gb300 import scene


def test_splitmix64_known_values():
    r = scene.SplitMix64(0)
    # splitmix64 from state 0 (Steele, Lea & Flood 2014): published first outputs
    assert r.next() == 0xE220A8397B1DCDAF
    assert r.next() == 0x6E789E6AA1B965F4


def test_scene_is_seeded_and_in_range():
    a = scene.make_scene(256, 0.9, 40, 5, 3)
    b = scene.make_scene(256, 0.9, 40, 5, 3)
    assert np.array_equal(a.boxes, b.boxes) and np.array_equal(a.spheres, b.spheres)
    assert (a.boxes[:, 2:4] >= 0.01).all() and (a.boxes[:, 2:4] <= 0.08).all()
    assert (a.boxes[:, 4] >= 0.2).all() and (a.boxes[:, 4] <= 0.85).all()
    c = scene.make_scene(256, 0.9, 40, 5, 4)
    assert not np.array_equal(a.boxes, c.boxes)


def test_box_covers_pixel_centres_inclusive():
    s = scene.Scene(n=8, plane=0.9, boxes=np.asarray([[0.5, 0.5, 0.1875, 0.0625, 0.3]], np.float32),
                    spheres=np.zeros((0, 4), np.float32))
    d = scene.rasterise(s)
    # centres (x+.5)/8: x=2..5 lie in [0.3125, 0.6875]; y=3,4 in [0.4375, 0.5625]
    want = np.full((8, 8), np.float32(0.9))
    want[3:5, 2:6] = np.float32(0.3)
    assert np.array_equal(d, want)


def test_sphere_depth_min_combines():
    s = scene.Scene(n=16, plane=0.95, boxes=np.zeros((0, 5), np.float32),
                    spheres=np.asarray([[0.5, 0.5, 0.2, 0.5]], np.float32))
    d = scene.rasterise(s)
    assert d.min() < 0.5 and d.max() == np.float32(0.95)
    assert d[8, 8] == d[7, 7]  # symmetric about the centre


def test_window_matches_full_raster():
    s = scene.make_scene(128, 0.95, 30, 6, 9)
    full = scene.rasterise(s)
    win = scene.rasterise(s, 32, 64, 64, 32)
    assert np.array_equal(win, full[64:96, 32:96])


def test_queries():
    q = scene.voxel_queries(1000, 64, 1)
    assert q.dtype == np.int32 and q.shape == (1000, 3) and q.min() >= 0 and q.max() < 64
    d = scene.rasterise(scene.make_scene(64, 0.9, 5, 0, 1))
    p = scene.ndc_queries_mixed(d, 1000, 2)
    assert p.dtype == np.float32 and p.shape == (1000, 3)
    assert np.abs(p[500:]).max() <= 1.0
