"""The oracle (C++ restatement, oracle/cpvs_oracle.cpp) against the
reference's own known answers and golden fixtures.  CPU only.

The known answers re-express the reference's unit tests
(test/MinMaxTest.cpp, test/CompressedShadowUtilTest.cpp,
test/CompressedShadowTest.cpp); the fixtures were written by the reference's
own build (tests/golden/make_golden.py).  Where the reference build exists
in this checkout (oracle/_ref), the restatement is also compared with it on
fresh seeded maps.
"""
import os

import numpy as np
import pytest

from oracle.oracle import REF_SO, split_pyramid

VIS, SH = 1, 0


def pyr_level(oracle, depth, level):
    return split_pyramid(oracle.pyramid(depth), depth.shape[0])[level - 1]


def to_ndc(v):
    """test/CompressedShadowTest.cpp:45-48: [0,1] -> [-1,1]."""
    return np.asarray(v, np.float32) * np.float32(2.0) + np.float32(-1.0)


def traverse(oracle, b, pts):
    return oracle.lookup_ndc(b.dag, b.num_levels, b.leafmasks, np.asarray(pts, np.float32).reshape(-1, 3))


# ---------------------------------------------------------------- MinMaxTest
def test_minmax_get_8x8(oracle, golden):
    img = golden["test_minmax_8x8_0/depth"]
    assert oracle.build(img).num_levels == 4                      # MinMaxTest.cpp:43
    l1, l2, l3 = (pyr_level(oracle, img, L) for L in (1, 2, 3))
    assert img[0, 0] == 0.0                                        # getMin/Max(0,0,0)
    assert l1[0, 0, 0] == np.float32(0.0) and l1[0, 0, 1] == np.float32(0.9)
    assert l2[0, 0, 1] == np.float32(1.0)
    assert l3[0, 0, 1] == np.float32(1.0) and l3[0, 0, 0] == np.float32(0.0)


def test_minmax_4x4(oracle, golden):
    img = golden["test_minmax_4x4_1/depth"]
    l1 = pyr_level(oracle, img, 1)
    assert l1[0, 0, 0] == 0.0 and l1[0, 0, 1] == 0.0 and l1[0, 1, 1] == 1.0   # MinMaxTest.cpp:68-70


def test_minmax_32x32(oracle, golden):
    img = golden["test_depths32x32/depth"]
    l4, l2 = pyr_level(oracle, img, 4), pyr_level(oracle, img, 2)
    close = lambda a, b: abs(float(a) - b) < 1e-6                  # MinMaxTest.cpp:73-75
    assert close(l4[1, 0, 0], 0.673203) and close(l4[0, 0, 0], 0.63008)
    assert close(l4[0, 1, 0], 0.63008) and close(l4[1, 1, 0], 0.700469)
    assert close(l2[1, 1, 0], 0.63008)


# ---------------------------------------------------- CompressedShadowUtilTest
def test_childmask_kat(oracle, golden):
    img = golden["test_depths8x8/depth"]
    assert oracle.child_mask(img, 1, 2, 0, 0) == 0x88AA            # CompressedShadowUtilTest.cpp:14-19
    assert int(golden["kat/childmask_8x8_l1_2_0_0"][0]) == 0x88AA


def test_merge_level_kat(oracle, golden):
    out, mapping, left = oracle.merge_level(golden["kat/merge_in"], 9)   # CompressedShadowUtilTest.cpp:67-97
    assert mapping[0] == 0 and mapping[1] == 9 and out[9] == 0xAAA0
    assert np.array_equal(out, golden["kat/merge_out"])
    assert np.array_equal(mapping, golden["kat/merge_mapping"])
    assert left == int(golden["kat/merge_left"][0]) == 2


# ---------------------------------------------------- CompressedShadowTest
def test_traverse_8x8(oracle, golden):
    b = oracle.build(golden["test_depths8x8/depth"])
    assert not b.leafmasks                                         # 4 levels: no leafmasks
    cases = [((-1, 1, -1), SH), ((-1, -1, 0), VIS), ((1, 1, 0), SH), ((0, 0, 0), SH), ((.5, .5, .5), SH),
             ((1, 1, -.75), VIS), ((1, 1, .5), SH), ((1, -1, .99), VIS), ((.7, -1, .99), SH),
             ((.45, -1, -.9), SH), ((.1, -1.0, -.9), SH)]            # CompressedShadowTest.cpp:50-88
    got = traverse(oracle, b, [c for c, _ in cases])
    assert got.tolist() == [v for _, v in cases]


def test_traverse_16x16(oracle, golden):
    b = oracle.build(golden["test_depths16x16/depth"])
    s = np.float32(2.0 / 16.0)
    cases = [((1, 1, 0), VIS), ((-1, -1, -1 + 3 * s), VIS), ((-1, -s, -1 + 3 * s), VIS), ((-1, 1, -1), SH),
             ((0, 0, -.9), VIS), ((0 + s, 0, .9), SH), ((0 + 3 * s, 0, -.9), VIS)]   # :90-117
    got = traverse(oracle, b, [c for c, _ in cases])
    assert got.tolist() == [v for _, v in cases]


def test_traverse_32x32(oracle, golden):
    b = oracle.build(golden["test_depths32x32/depth"])
    s = 2.0 / 32.0
    cases = [((1, 1, 0), VIS), ((-1 + 7 * s, 1 - 7 * s, .5), VIS), ((-1 + 7 * s, 1 - 7 * s, .6), SH),
             ((-1 + 7 * s, -1 + 8 * s, .3), SH)]                    # :119-136
    assert traverse(oracle, b, [c for c, _ in cases]).tolist() == [v for _, v in cases]
    lit = [to_ndc((x / 32.0, y / 32.0, 0.59)) for y in range(31) for x in range(31)]       # :138-144
    assert (traverse(oracle, b, lit) == VIS).all()
    dark = [to_ndc((x / 32.0, y / 32.0, 0.79)) for y in range(8, 26) for x in range(7, 27)]  # :145-151
    assert (traverse(oracle, b, dark) == SH).all()


# ------------------------------------------------------------ golden fixtures
def test_oracle_matches_reference_fixtures(oracle, golden, golden_cases):
    seen = set()
    for key in golden_cases:
        name, zt = key.split("/")
        zi, zn = (int(v) for v in zt[1:].split("of"))
        depth = golden[f"{name}/depth"]
        if name not in seen:
            seen.add(name)
            assert np.array_equal(oracle.pyramid(depth).view(np.uint32), golden[f"{name}/pyramid"].view(np.uint32)), name
        b = oracle.build(depth, zi, zn)
        nl, tv, lm = golden[f"{key}/meta"].tolist()
        assert b.ref_defined
        assert b.num_levels == nl and b.leafmasks == bool(lm), key
        assert np.array_equal(b.dag, golden[f"{key}/dag"]), key
        assert int(oracle.lib.oracle_total_visibility(b.dag)) == tv, key
        vis = oracle.lookup_ndc(b.dag, b.num_levels, b.leafmasks, golden[f"{name}/ndc"])
        assert np.array_equal(vis, golden[f"{key}/vis"]), key


def test_pyramid_only_fixtures(oracle, golden):
    """Maps too small for a DAG still have a reference pyramid (4x4)."""
    d = golden["test_minmax_4x4_1/depth"]
    assert np.array_equal(oracle.pyramid(d).view(np.uint32), golden["test_minmax_4x4_1/pyramid"].view(np.uint32))


def test_linear_merge_equals_hash_merge(oracle):
    from cpvs_gb300 import scene
    d = scene.rasterise(scene.make_scene(128, 0.9, 15, 2, 5))
    a = oracle.build(d)
    b = oracle.build(d, linear_merge=True)
    assert np.array_equal(a.dag, b.dag)


def test_undefined_reference_case_is_flagged(oracle):
    """An SVO that ends above its leaf level makes the reference read past
    its array (levelExists, src/CompressedShadow.cpp:208-213); the oracle
    flags it and still builds the intended DAG."""
    b = oracle.build(np.full((64, 64), 0.25, np.float32))
    assert not b.ref_defined
    # root: 4 partial children, all the same node, which is lit above / shadowed below
    assert b.dag.tolist() == [0xAA, 5, 5, 5, 5, 0x55]
    assert oracle.build(np.full((64, 64), 0.3, np.float32)).ref_defined


def test_grid_lookup_restatement_routes_cells(oracle):
    """Two z-tiles of one map in a 1x1x2... grid must answer like each tile's
    own lookup on local coordinates."""
    from cpvs_gb300 import scene
    d = scene.rasterise(scene.make_scene(64, 0.9, 8, 1, 3))
    L = 2
    dags, offs, off = [], [], 0
    tiles = {}
    for z in range(L):
        b = oracle.build(d, z, L)
        tiles[z] = b
    # a grid of length 2 needs 8 cells: reuse the z-tile DAGs for both x,y
    for cz in range(L):
        for cy in range(L):
            for cx in range(L):
                b = tiles[cz]
                dags.append(b.dag)
                offs.append(off)
                off += b.dag.size
    dag = np.concatenate(dags).astype(np.uint32)
    rng = np.random.default_rng(0)
    q = rng.uniform(-1, 1, (5000, 3)).astype(np.float32)
    got = oracle.grid_lookup_ndc(dag, np.asarray(offs, np.uint32), L, tiles[0].num_levels, True, q)
    res = (1 << (tiles[0].num_levels + 1 - 1)) - 1
    p = (((q + np.float32(1)) * np.float32(0.5)) * np.float32(res)).astype(np.int32)
    n = 64
    for z in range(L):
        sel = (p[:, 2] // n) == z
        local = p[sel] % n
        want = oracle.lookup_voxel(tiles[z].dag, tiles[z].num_levels, True, local)
        assert np.array_equal(got[sel], want)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference build not present in this checkout")
def test_oracle_matches_reference_build_fresh_maps(oracle):
    from oracle.oracle import Reference
    from cpvs_gb300 import scene
    R = Reference()
    rng = np.random.default_rng(99)
    for trial in range(60):
        n = int(rng.choice([8, 16, 32, 64, 128]))
        kind = trial % 4
        if kind == 0:
            d = rng.random((n, n), dtype=np.float32)
        elif kind == 1:
            d = (rng.integers(0, 8, (n, n)) / 7).astype(np.float32)
        elif kind == 2:
            d = scene.rasterise(scene.make_scene(n, 0.9, int(rng.integers(1, 12)), 2, int(rng.integers(1 << 30))))
        else:
            d = (rng.random((n, n)) * 0.2 + 0.7).astype(np.float32)
        zn = int(rng.choice([1, 2, 3, 4]))
        zi = int(rng.integers(0, zn))
        b = oracle.build(d, zi, zn)
        if not b.ref_defined:
            continue
        q = rng.uniform(-1, 1, (2000, 3)).astype(np.float32)
        dag, nl, tv, vis = R.create(d, zi, zn, ndc=q, try_leafmasks=n >= 16)
        assert nl == b.num_levels
        assert np.array_equal(dag, b.dag), (trial, n, zi, zn)
        assert np.array_equal(vis, oracle.lookup_ndc(b.dag, b.num_levels, b.leafmasks, q))


def _all_voxels(n):
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.int32)


@pytest.mark.parametrize("kind", ["uniform", "scene", "quantised"])
def test_every_voxel_answer_is_the_direct_depth_test(oracle, kind):
    """A size-independent property of the whole build: every voxel's answer
    from the DAG equals the per-voxel test of cs::absoluteVisible
    (src/CompressedShadowUtil.h:51-57) applied to the map directly -- lit iff
    the float32 voxel centre (Z + (Z+1)) * 0.5 <= fl(d * n * zTileNum) for the
    global voxel height Z = z + t*n of z-tile t.  It holds exactly because a
    level's height is the map's divided by a power of two, so the min/max
    classification of an inner node never contradicts its voxels."""
    from cpvs_gb300 import scene
    n = 64
    g = np.random.default_rng(11)
    if kind == "uniform":
        d = g.uniform(0, 1, (n, n)).astype(np.float32)
    elif kind == "scene":
        d = scene.rasterise(scene.make_scene(n, 0.9, 10, 2, 3))
    else:
        d = (np.floor(g.uniform(0, 1, (n, n)) * n) / n).astype(np.float32)
    q = _all_voxels(n)
    f32 = np.float32
    for K, leaf in ((1, True), (4, True), (1, False), (2, False)):
        for t in range(K):
            b = oracle.build(d, t, K, leafmasks=leaf)
            got = oracle.lookup_voxel(b.dag, b.num_levels, b.leafmasks, q)
            Z = q[:, 2].astype(np.int64) + t * n
            mid = (Z.astype(f32) + (Z + 1).astype(f32)) * f32(0.5)
            dh = d[q[:, 1], q[:, 0]].astype(f32) * f32(n * K)
            want = np.where(mid <= dh, 1, 0)
            assert np.array_equal(got, want), (kind, K, t, leaf)


def _walk_dag(dag, num_levels, leafmasks):
    """Parses a DAG from its root, level by level: returns per level the node
    offsets and words, after checking the reference's layout
    (src/CompressedShadow.cpp:306-392): each level's nodes lie back to back,
    levels follow each other top-down from word 0, and a level's nodes are in
    the order of their first reference from the level above (parents in
    order, children in index order)."""
    levels = {}
    frontier, L, expect = [0], num_levels - 2, 0
    while frontier:
        nodes, refs = [], []
        for off in frontier:
            assert off == expect, ("level not contiguous", L, off, expect)
            m = int(dag[off])
            k = bin(m & 0xAAAA).count("1")
            leaf = leafmasks and L == 2
            size = 1 + (2 * k if leaf else k)
            words = tuple(int(w) for w in dag[off:off + size])
            nodes.append(words)
            if not leaf:
                refs.extend(words[1:])
            expect = off + size
        levels[L] = nodes
        first = list(dict.fromkeys(refs))  # first-occurrence order
        assert first == sorted(first), ("children not in first-occurrence order", L)
        frontier, L = first, L - 1
    assert expect == len(dag), ("words outside the reachable nodes", expect, len(dag))
    return levels


@pytest.mark.parametrize("leaf", [True, False])
def test_dag_is_minimal_and_laid_out_as_the_reference(oracle, leaf):
    """No two nodes of a level are equal (the merge is complete), every word
    belongs to a reachable node, and the per-level node counts are the
    unique counts the build reports."""
    from cpvs_gb300 import scene
    g = np.random.default_rng(2)
    maps = [g.uniform(0, 1, (64, 64)).astype(np.float32),
            scene.rasterise(scene.make_scene(256, 0.9, 40, 4, 12)),
            (np.floor(g.uniform(0, 1, (128, 128)) * 8) / 8).astype(np.float32)]
    for d in maps:
        for t, K in ((0, 1), (1, 2)):
            b = oracle.build(d, t, K, leafmasks=leaf)
            if not b.ref_defined:
                continue
            levels = _walk_dag(b.dag, b.num_levels, b.leafmasks)
            for L, nodes in levels.items():
                assert len(set(nodes)) == len(nodes), ("duplicate nodes", L)
                assert len(nodes) == b.unique_nodes[L], (L, len(nodes), b.unique_nodes[L])


def test_reference_dags_have_the_layout_the_walker_checks(golden, golden_cases):
    """The same layout and minimality checks hold for every DAG the
    reference itself wrote into the golden fixtures, so they restate the
    reference's format rather than the oracle's."""
    for key in golden_cases:
        nl, _tv, lm = golden[f"{key}/meta"].tolist()
        levels = _walk_dag(golden[f"{key}/dag"], nl, bool(lm))
        for L, nodes in levels.items():
            assert len(set(nodes)) == len(nodes), (key, L)


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["c0", "c1"])
def test_oracle_matches_reference_at_config_scale(oracle, golden_configs, name):
    """The benchmarked workloads themselves (1024^2, 40 boxes; 8192^2, 500
    boxes and 64 spheres), against what the reference's own create and
    traverse wrote (tests/golden/make_golden_configs.py): the DAG (words at
    1024^2, length and SHA-256 at 8192^2), per-level tree and unique node
    counts, numLevels, and the answers on 2^16 mixed NDC points."""
    from cpvs_gb300 import scene
    g = golden_configs
    d = scene.rasterise(scene.config_scene(name))
    assert _sha(d) == str(g[f"{name}/map_sha256"]), "the scene generator no longer reproduces the map"
    b = oracle.build(d, threads=4)
    nl, tv, words = g[f"{name}/meta"].tolist()
    assert b.num_levels == nl and b.dag.size == words
    assert _sha(b.dag) == str(g[f"{name}/dag_sha256"])
    if name == "c0":
        assert np.array_equal(b.dag, g["c0/dag"])
    assert list(b.unique_nodes) == g[f"{name}/unique_nodes"].tolist()
    assert list(b.tree_nodes) == g[f"{name}/tree_nodes"].tolist()
    q = scene.ndc_queries_mixed(d, 1 << 16, int(g[f"{name}/ndc_seed"]))
    assert _sha(q) == str(g[f"{name}/ndc_sha256"])
    assert np.array_equal(oracle.lookup_ndc(b.dag, nl, True, q, threads=4), g[f"{name}/ndc_vis"])
    if name == "c0":
        v = scene.voxel_queries(1 << 20, 1024, 0)[:1 << 16]
        assert _sha(v) == str(g["c0/voxel_sha256"])
        assert np.array_equal(oracle.lookup_voxel(b.dag, nl, True, v, threads=4), g["c0/voxel_vis"])
