"""Seeded synthetic shadow scenes: depth maps under an orthographic light and
light-space query sets.

Input synthesis only (not the shadow hot path).  The reference renders its
shadow map with OpenGL (src/DeferredRenderer.cpp:124-148); here a scene is a
ground plane plus axis-aligned boxes and spheres, rasterised to a float32
depth map on the host with numpy.  The same primitives can be rasterised on
the device by ``cpvs_raster_depth`` in the CUDA library, which follows the
float32 operation order used below bit for bit.

Random draws come from splitmix64 (Steele, Lea & Flood 2014), which is
trivially identical in Python, C++ and CUDA; a uniform draw is the top 24 bits
of one output scaled by 2**-24, exact in float32.
"""
from __future__ import annotations

import dataclasses

import numpy as np

_MASK = (1 << 64) - 1


class SplitMix64:
    """splitmix64: state += golden gamma, then two xor-shift-multiply rounds."""

    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return float(self.next() >> 40) * (2.0 ** -24)

    def uniform_in(self, lo: float, hi: float) -> np.float32:
        return np.float32(lo + (hi - lo) * self.uniform())


@dataclasses.dataclass
class Scene:
    """Primitives of one depth map.  Boxes: (cx, cy, hx, hy, top); spheres:
    (cx, cy, r, centre_depth).  Coordinates are in [0,1] over the map."""

    n: int
    plane: float
    boxes: np.ndarray    # (nb, 5) float32
    spheres: np.ndarray  # (ns, 4) float32


def make_scene(n: int, plane: float, n_boxes: int, n_spheres: int, seed: int,
               half_extent=(0.01, 0.08), top=(0.2, 0.85),
               radius=(0.005, 0.05), centre_depth=(0.2, 0.85)) -> Scene:
    """Draw order per box: cx, cy, hx, hy, top; per sphere: cx, cy, r, depth."""
    rng = SplitMix64(seed)
    boxes = np.zeros((n_boxes, 5), np.float32)
    for i in range(n_boxes):
        boxes[i] = (rng.uniform_in(0, 1), rng.uniform_in(0, 1), rng.uniform_in(*half_extent),
                    rng.uniform_in(*half_extent), rng.uniform_in(*top))
    spheres = np.zeros((n_spheres, 4), np.float32)
    for i in range(n_spheres):
        spheres[i] = (rng.uniform_in(0, 1), rng.uniform_in(0, 1), rng.uniform_in(*radius),
                      rng.uniform_in(*centre_depth))
    return Scene(n=n, plane=float(np.float32(plane)), boxes=boxes, spheres=spheres)


# The workloads of the benchmark and the parity tests (sizes from the
# reference's use: 1024^2 single map, 8192^2 single map (its tile cap,
# src/DeferredRenderer.cpp:189-200), 32768^2 split into 4096^2 tiles).
CONFIGS = {
    "c0": dict(n=1024, plane=0.9, n_boxes=40, n_spheres=0, seed=0),
    "c1": dict(n=8192, plane=0.95, n_boxes=500, n_spheres=64, seed=1),
    "c2": dict(n=32768, plane=0.95, n_boxes=4000, n_spheres=512, seed=2),
}


def config_scene(name: str, n: int | None = None) -> Scene:
    c = dict(CONFIGS[name])
    if n is not None:
        c["n"] = n
    return make_scene(**c)


def pixel_centres(n: int) -> np.ndarray:
    """(x + 0.5) / n in float32; exact for power-of-two n."""
    return ((np.arange(n, dtype=np.float32) + np.float32(0.5)) / np.float32(n)).astype(np.float32)


def rasterise(scene: Scene, x0: int = 0, y0: int = 0, w: int | None = None, h: int | None = None) -> np.ndarray:
    """Depth map (rows y, columns x) of a scene, or of the window
    [x0,x0+w) x [y0,y0+h) of it.  A box covers the pixels whose centre lies in
    [c-h, c+h] on both axes and min-combines its top depth.  A sphere
    min-combines centre_depth - sqrt(r*r - rho2) where rho2 = dx*dx + dy*dy < r*r,
    all in float32 with that operation order."""
    n = scene.n
    w = n if w is None else w
    h = n if h is None else h
    cx_all = pixel_centres(n)
    xs, ys = cx_all[x0:x0 + w], cx_all[y0:y0 + h]
    depth = np.full((h, w), np.float32(scene.plane), np.float32)
    for cx, cy, hx, hy, top in scene.boxes:
        lox, hix = np.float32(cx - hx), np.float32(cx + hx)
        loy, hiy = np.float32(cy - hy), np.float32(cy + hy)
        ax, bx = np.searchsorted(xs, lox, "left"), np.searchsorted(xs, hix, "right")
        ay, by = np.searchsorted(ys, loy, "left"), np.searchsorted(ys, hiy, "right")
        if ax < bx and ay < by:
            sub = depth[ay:by, ax:bx]
            np.minimum(sub, top, out=sub)
    for cx, cy, r, dc in scene.spheres:
        lox, hix = np.float32(cx - r), np.float32(cx + r)
        loy, hiy = np.float32(cy - r), np.float32(cy + r)
        ax, bx = np.searchsorted(xs, lox, "left"), np.searchsorted(xs, hix, "right")
        ay, by = np.searchsorted(ys, loy, "left"), np.searchsorted(ys, hiy, "right")
        if not (ax < bx and ay < by):
            continue
        dx = (xs[ax:bx] - cx).astype(np.float32)
        dy = (ys[ay:by] - cy).astype(np.float32)
        rho2 = (dy[:, None] * dy[:, None]) + (dx[None, :] * dx[None, :])
        r2 = np.float32(r * r)
        inside = rho2 < r2
        hgt = np.sqrt(np.where(inside, r2 - rho2, np.float32(0)).astype(np.float32))
        d = (np.float32(dc) - hgt).astype(np.float32)
        sub = depth[ay:by, ax:bx]
        np.minimum(sub, np.where(inside, d, sub), out=sub)
    return depth


def voxel_queries(count: int, n: int, seed: int) -> np.ndarray:
    """count x 3 int32 voxel coordinates uniform in [0, n)^3."""
    g = np.random.Generator(np.random.PCG64(seed))
    return g.integers(0, n, size=(count, 3), dtype=np.int32)


def ndc_queries_mixed(depth: np.ndarray, count: int, seed: int) -> np.ndarray:
    """count x 3 float32 light-space (NDC) points: the first half on the depth
    surface (pixel centre, z = depth*n offset uniformly by up to half a voxel),
    the second half uniform in [-1,1]^3.  Voxel v maps to NDC 2v/(n-1)-1, the
    inverse of the reference's quantisation (src/CompressedShadowUtil.h:70-75)."""
    n = depth.shape[0]
    g = np.random.Generator(np.random.PCG64(seed))
    half = count // 2
    out = np.empty((count, 3), np.float32)
    px = g.integers(0, n, size=half)
    py = g.integers(0, n, size=half)
    vz = depth[py, px].astype(np.float64) * n + (g.random(half) - 0.5)
    scale = 2.0 / (n - 1)
    out[:half, 0] = (px + 0.5) * scale - 1.0
    out[:half, 1] = (py + 0.5) * scale - 1.0
    out[:half, 2] = vz * scale - 1.0
    out[half:] = (g.random((count - half, 3)) * 2.0 - 1.0).astype(np.float32)
    return out


def rasterise_triangles(tris: np.ndarray, n: int, plane: float, x0: int = 0, y0: int = 0, w: int | None = None,
                        h: int | None = None) -> np.ndarray:
    """Host rasteriser for (m, 9) float32 triangles (x0,y0,d0, x1,y1,d1,
    x2,y2,d2 in map coordinates [0,1]) over a plane: the rule of
    cpvs_raster_triangles (include/cpvs.h) -- pixel centre inside the bounding
    box, edge functions with the sign of the area, depth
    ((e0 d0 + e1 d1) + e2 d2) / area -- in float32, round to nearest, in that
    operation order; each pixel keeps the minimum (NaN propagates)."""
    w = n if w is None else w
    h = n if h is None else h
    f = np.float32
    cx_all = pixel_centres(n)
    xs, ys = cx_all[x0:x0 + w], cx_all[y0:y0 + h]
    depth = np.full((h, w), f(plane), f)
    tris = np.asarray(tris, f).reshape(-1, 9)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        for t in tris:
            X0, Y0, D0, X1, Y1, D1, X2, Y2, D2 = (f(v) for v in t)
            if np.isnan([X0, Y0, X1, Y1, X2, Y2]).any():
                continue
            minx, maxx = min(X0, X1, X2), max(X0, X1, X2)
            miny, maxy = min(Y0, Y1, Y2), max(Y0, Y1, Y2)
            ax = np.searchsorted(xs, minx, "left")
            bx = np.searchsorted(xs, maxx, "right")
            ay = np.searchsorted(ys, miny, "left")
            by = np.searchsorted(ys, maxy, "right")
            if ax >= bx or ay >= by:
                continue
            px = xs[ax:bx][None, :]
            py = ys[ay:by][:, None]
            e0 = (f(X2 - X1) * (py - Y1)) - (f(Y2 - Y1) * (px - X1))
            e1 = (f(X0 - X2) * (py - Y2)) - (f(Y0 - Y2) * (px - X2))
            e2 = (f(X1 - X0) * (py - Y0)) - (f(Y1 - Y0) * (px - X0))
            area = (e0 + e1) + e2
            inside = ((area > 0) & (e0 >= 0) & (e1 >= 0) & (e2 >= 0)) | \
                     ((area < 0) & (e0 <= 0) & (e1 <= 0) & (e2 <= 0))
            v = (((e0 * D0) + (e1 * D1)) + (e2 * D2)) / area
            sub = depth[ay:by, ax:bx]
            np.minimum(sub, np.where(inside, v, sub).astype(f), out=sub)
    return depth


def terrain_triangles(cells: int, seed: int, lo: float = 0.3, hi: float = 0.8) -> np.ndarray:
    """A height-field mesh: a cells x cells grid of quads over [0,1]^2, each
    split into two triangles sharing an edge, vertex depths uniform in
    [lo, hi) (seeded); (2 cells^2, 9) float32."""
    g = np.random.Generator(np.random.PCG64(seed))
    hgt = (lo + (hi - lo) * g.random((cells + 1, cells + 1))).astype(np.float32)
    c = np.linspace(0.0, 1.0, cells + 1, dtype=np.float32)
    out = []
    for j in range(cells):
        for i in range(cells):
            a = (c[i], c[j], hgt[j, i])
            b = (c[i + 1], c[j], hgt[j, i + 1])
            d = (c[i], c[j + 1], hgt[j + 1, i])
            e = (c[i + 1], c[j + 1], hgt[j + 1, i + 1])
            out.append((*a, *b, *e))
            out.append((*a, *e, *d))
    return np.asarray(out, np.float32)
