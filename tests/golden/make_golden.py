"""Writes tests/golden/reference_fixtures.npz from the reference itself.

Run in a checkout where the reference is present (it is read, never
modified):

    make -C oracle ref            # the reference's own CPU build, in place
    python tests/golden/make_golden.py [/path/to/reference]   # default: $CPVS_REFERENCE_DIR

Inputs:
  * the depth images of the reference's unit tests, parsed from
    test/TestImages.cpp (depths8x8/16x16/32x32) and test/MinMaxTest.cpp (the
    inline 8x8 and 4x4 images);
  * seeded synthetic maps (scene rasteriser of cpvs_gb300.scene, uniform
    noise, quantised depths, signed zeros), some built as z-tiles.
Outputs per case: the reference's pyramid, DAG words, numLevels, total
visibility and CompressedShadow::traverse results for a fixed set of NDC
points.  The GPU parity tests and the oracle tests compare against these
without needing the reference at run time.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cpvs_gb300 import scene  # noqa: E402
from oracle.oracle import Oracle, Reference  # noqa: E402

OUT = os.path.join(HERE, "reference_fixtures.npz")


def parse_float_list(body: str) -> np.ndarray:
    vals = [float(v) for v in re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", body)]
    return np.asarray(vals, np.float32)


def reference_test_images(ref_dir: str) -> dict:
    imgs = {}
    src = open(os.path.join(ref_dir, "test", "TestImages.cpp")).read()
    for name in ("depths8x8", "depths16x16", "depths32x32"):
        m = re.search(name + r"\s*\{(.*?)\};", src, re.S)
        a = parse_float_list(m.group(1))
        n = int(round(np.sqrt(a.size)))
        imgs["test_" + name] = a.reshape(n, n)
    mm = open(os.path.join(ref_dir, "test", "MinMaxTest.cpp")).read()
    bodies = re.findall(r"setAll\((?:std::)?vector<float>\s*\{(.*?)\}\)", mm, re.S)
    for k, body in enumerate(bodies):
        a = parse_float_list(body)
        n = int(round(np.sqrt(a.size)))
        imgs[f"test_minmax_{n}x{n}_{k}"] = a.reshape(n, n)
    return imgs


def ndc_probe_points(n_side: int, rng: np.random.Generator) -> np.ndarray:
    g = np.linspace(-1.0, 1.0, n_side, dtype=np.float32)
    grid = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rnd = rng.uniform(-1.0, 1.0, (4096, 3)).astype(np.float32)
    return np.concatenate([grid, rnd]).astype(np.float32)


def main(ref_dir: str):
    R = Reference()
    O = Oracle()
    rng = np.random.default_rng(20240601)
    cases = dict(reference_test_images(ref_dir))
    # seeded synthetic maps
    for n, seed in ((64, 11), (128, 12), (256, 13)):
        cases[f"scene{n}"] = scene.rasterise(scene.make_scene(n, 0.9, 12, 3, seed))
    cases["noise64"] = rng.random((64, 64), dtype=np.float32)
    cases["quantised128"] = (rng.integers(0, 16, (128, 128)) / 15.0).astype(np.float32)
    sz = rng.random((32, 32), dtype=np.float32) * 0.5 + 0.25
    sz[rng.random((32, 32)) < 0.2] = -0.0
    sz[rng.random((32, 32)) < 0.2] = 0.0
    cases["signed_zero32"] = sz.astype(np.float32)
    cases["const_lit16"] = np.ones((16, 16), np.float32)
    cases["const_shadow16"] = np.zeros((16, 16), np.float32)
    cases["noise8"] = rng.random((8, 8), dtype=np.float32)

    ztiles = {"scene128": 4, "scene64": 3, "test_depths32x32": 2}
    out = {}
    names = []
    for name, depth in cases.items():
        depth = np.ascontiguousarray(depth, np.float32)
        n = depth.shape[0]
        pts = ndc_probe_points(9 if n <= 16 else 13, rng)
        # the reference builds DAGs only for numLevels > 3 (src/CompressedShadow.cpp:46)
        tiles = [(0, 1)] + [(i, ztiles[name]) for i in range(ztiles.get(name, 0))] if n >= 8 else []
        out[f"{name}/depth"] = depth
        out[f"{name}/pyramid"] = R.pyramid(depth)
        out[f"{name}/ndc"] = pts
        for zi, zn in tiles:
            if not O.build(depth, zi, zn).ref_defined:
                print(f"skip {name} z{zi}/{zn}: the reference's build is undefined there")
                continue
            dag, nl, tv, vis = R.create(depth, zi, zn, ndc=pts, try_leafmasks=(nl_ok := n >= 16))
            key = f"{name}/z{zi}of{zn}"
            out[f"{key}/dag"] = dag
            out[f"{key}/meta"] = np.asarray([nl, tv, int(nl_ok)], np.int64)
            out[f"{key}/vis"] = vis
            names.append(key)
    # reference unit-test KATs that are functions, not builds
    out["kat/childmask_8x8_l1_2_0_0"] = np.asarray(
        [R.child_mask(cases["test_depths8x8"], 1, 2, 0, 0)], np.uint32)
    merge_in = np.asarray([0xAAAA, 10, 42, 0, 0, 1, 2, 3, 4,
                           0xAAA0, 10, 0, 0, 0, 0, 0, 0, 0,
                           0xAAAA, 10, 42, 0, 0, 1, 2, 3, 4], np.uint32)
    merged, mapping, left = R.merge_level(merge_in, 9)
    out["kat/merge_in"] = merge_in
    out["kat/merge_out"] = merged
    out["kat/merge_mapping"] = mapping
    out["kat/merge_left"] = np.asarray([left], np.int64)
    out["kat/grid_levels"] = np.asarray([R.grid_levels(L ** 3) for L in (1, 2, 4, 8, 16)], np.int64)
    out["index/cases"] = np.asarray(names)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {len(names)} builds, {os.path.getsize(OUT) // 1024} KiB")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CPVS_REFERENCE_DIR", "/root/reference"))
