"""Writes tests/golden/reference_configs.npz: the reference's own answers on
the two benchmarked plain-method workloads, the 1024^2 map of 40 boxes and
the 8192^2 map of 500 boxes and 64 spheres.

Run where the reference checkout is present (it is read, never modified):

    make -C oracle ref REF_DIR=...      # the reference's own CPU build, in place
    CPVS_REFERENCE_DIR=... python tests/golden/make_golden_configs.py

It runs the reference's CompressedShadow::create (src/CompressedShadow.cpp:49-59)
on each map and CompressedShadow::traverse (:404-463) on a fixed set of NDC
points, through oracle/_ref (the reference's sources compiled unmodified).
The 8192^2 build takes several minutes, because the reference's merge scans
every kept node of a level for each node (src/CompressedShadowUtil.h:154-182).

Stored per workload:
  * the SHA-256 of the depth map (the synthetic generator in
    cpvs_gb300/scene.py must reproduce it bit for bit);
  * numLevels and the total visibility;
  * the DAG itself for the 1024^2 map (about 62 KB), and for the 8192^2 map
    its length and SHA-256 (9 MB is too large to commit);
  * per level, the tree node count and the unique node count, found by
    walking the reference's DAG from the root (tree counts are path counts);
  * the reference's traverse answers on 2^16 mixed surface/volume NDC points
    (cpvs_gb300.scene.ndc_queries_mixed with the seed stored here) and, for
    the 1024^2 map, on the voxel centres of the first 2^16 of its 2^20 voxel
    queries (cpvs_gb300.scene.voxel_queries), with the SHA-256 of each point
    set so a test can tell a drifted generator from a wrong answer.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cpvs_gb300 import scene  # noqa: E402
from oracle.oracle import Reference  # noqa: E402

OUT = os.path.join(HERE, "reference_configs.npz")
NQ = 1 << 16


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def voxel_centre_ndc(v: np.ndarray, n: int) -> np.ndarray:
    """NDC points that the reference's getPathFromNDC
    (src/CompressedShadowUtil.h:70-75) quantises to the voxels `v`."""
    return ((v.astype(np.float64) + 0.5) * (2.0 / (n - 1)) - 1.0).astype(np.float32)


def quantise(ndc: np.ndarray, n: int) -> np.ndarray:
    """getPathFromNDC in float32: ((ndc + 1) * 0.5) * (n - 1), truncated."""
    f = np.float32
    t = (ndc.astype(f) + f(1.0)).astype(f)
    t = (t * f(0.5)).astype(f)
    return np.trunc((t * f(n - 1)).astype(f)).astype(np.int64)


def walk_counts(dag: np.ndarray, num_levels: int, leafmasks: bool):
    """Per level (index = level), the unique node count and the tree node
    count of a DAG in the reference's layout: levels top-down from the root
    at word 0, inner node = mask + k absolute child offsets, leaf (level 2
    with leafmasks) = mask + 2k leafmask words.  A node's tree count is the
    number of root paths that reach it."""
    uniq = [0] * num_levels
    tree = [0] * num_levels
    frontier = {0: 1}
    L = num_levels - 2
    while frontier and L >= 0:
        uniq[L] = len(frontier)
        tree[L] = sum(frontier.values())
        leaf = leafmasks and L == 2
        nxt: dict = {}
        if not leaf:
            for off in sorted(frontier):
                m = int(dag[off])
                k = bin(m & 0xAAAA).count("1")
                mult = frontier[off]
                for c in dag[off + 1:off + 1 + k].tolist():
                    nxt[c] = nxt.get(c, 0) + mult
        frontier = nxt
        L -= 1
    return np.asarray(uniq, np.int64), np.asarray(tree, np.int64)


def main() -> None:
    R = Reference()
    out = {}
    for name, nq_seed in (("c0", 0), ("c1", 1)):
        t0 = time.time()
        d = scene.rasterise(scene.config_scene(name))
        n = d.shape[0]
        q = scene.ndc_queries_mixed(d, NQ, nq_seed)
        pts = [q]
        if name == "c0":
            v = scene.voxel_queries(1 << 20, n, 0)[:NQ]
            qv = voxel_centre_ndc(v, n)
            assert np.array_equal(quantise(qv, n), v), "voxel-centre NDC points do not quantise back"
            pts.append(qv)
        allq = np.concatenate(pts)
        dag, nl, tv, vis = R.create(d, 0, 1, ndc=allq, try_leafmasks=True)
        uniq, tree = walk_counts(dag, nl, True)
        out[f"{name}/map_sha256"] = np.asarray(sha(d))
        out[f"{name}/meta"] = np.asarray([nl, tv, dag.size], np.int64)
        out[f"{name}/dag_sha256"] = np.asarray(sha(dag))
        out[f"{name}/unique_nodes"] = uniq
        out[f"{name}/tree_nodes"] = tree
        out[f"{name}/ndc_seed"] = np.asarray(nq_seed, np.int64)
        out[f"{name}/ndc_sha256"] = np.asarray(sha(q))
        out[f"{name}/ndc_vis"] = vis[:NQ]
        if name == "c0":
            out["c0/dag"] = dag
            out["c0/voxel_sha256"] = np.asarray(sha(v))
            out["c0/voxel_vis"] = vis[NQ:]
        print(f"{name}: {n}^2 map, DAG {dag.size} words, levels {nl}, unique {uniq.tolist()}, "
              f"{time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {os.path.getsize(OUT) // 1024} KiB")


if __name__ == "__main__":
    main()
