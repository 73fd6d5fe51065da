"""GPU parity: the CUDA path, called through the C ABI, against the
reference's golden fixtures and the oracle.  Integer/bit work: every
comparison is exact (DAG words, pyramid bits, visibility bits)."""
import numpy as np
import pytest

from cpvs_gb300 import scene

pytestmark = pytest.mark.gpu


def split_key(key):
    name, zt = key.split("/")
    zi, zn = (int(v) for v in zt[1:].split("of"))
    return name, zi, zn


def hierarchy_levels(cp, mm):
    return np.concatenate([mm.level(L).reshape(-1) for L in range(1, mm.get_num_levels())])


# ------------------------------------------------------------ golden fixtures
def test_pyramid_matches_reference(cp, golden, golden_cases):
    names = sorted({k.split("/")[0] for k in golden_cases} | {"test_minmax_4x4_1"})
    for name in names:
        depth = golden[f"{name}/depth"]
        mm = cp.MinMaxHierarchy(depth)
        assert mm.get_num_levels() == int(np.log2(depth.shape[0])) + 1
        got = hierarchy_levels(cp, mm)
        assert np.array_equal(got.view(np.uint32), golden[f"{name}/pyramid"].view(np.uint32)), name


def test_device_map_pyramid_equals_host_map_pyramid(cp):
    """A map in device memory is reduced where it lies, a host map by the
    pass that also copies it as it reads it: both give the same bits, signed
    zeros, infinities and NaN included (the NaN flag too, through the DAG)."""
    torch = pytest.importorskip("torch")
    g = np.random.Generator(np.random.PCG64(17))
    for n in (64, 128, 256, 1024, 4096):
        d = g.random((n, n)).astype(np.float32)
        k = max(n * n // 50, 4)
        idx = g.integers(0, n * n, size=(4, k))
        flat = d.reshape(-1)
        flat[idx[0]] = -0.0
        flat[idx[1]] = 0.0
        flat[idx[2]] = np.inf if n % 2 == 0 else -np.inf
        if n != 1024:
            flat[idx[3]] = np.nan  # one size without NaN keeps the min/max shortcut on
        host = hierarchy_levels(cp, cp.MinMaxHierarchy(d))
        dev = hierarchy_levels(cp, cp.MinMaxHierarchy(torch.from_numpy(d).cuda()))
        assert np.array_equal(host.view(np.uint32), dev.view(np.uint32)), n
        a = cp.CompressedShadow.from_depth(d).get_dag()
        b = cp.CompressedShadow.from_depth(torch.from_numpy(d).cuda()).get_dag()
        assert np.array_equal(a, b), n


def test_hierarchy_batch_equals_single_hierarchies(cp):
    """cpvs_hierarchy_create_batch over maps of many sides (one launch per
    pass for all of them) gives each map the pyramid of its own
    cpvs_hierarchy_create, bit for bit, from host or device maps, and the
    same DAGs (so the same NaN flags)."""
    torch = pytest.importorskip("torch")
    g = np.random.Generator(np.random.PCG64(23))
    sides = [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 64, 8, 256]
    maps = []
    for i, n in enumerate(sides):
        d = g.random((n, n)).astype(np.float32)
        flat = d.reshape(-1)
        k = max(n * n // 40, 1)
        flat[g.integers(0, n * n, k)] = (-0.0, 0.0, np.inf, -np.inf, np.nan)[i % 5]
        maps.append(d)
    single = [hierarchy_levels(cp, cp.MinMaxHierarchy(d)) for d in maps]
    for kind in ("host", "device", "borrow"):
        src = maps if kind == "host" else [torch.from_numpy(d).cuda() for d in maps]
        hs = cp.MinMaxHierarchy.create_batch(src, borrow=kind == "borrow")
        assert len(hs) == len(maps)
        for i, h in enumerate(hs):
            assert h.get_num_levels() == int(np.log2(sides[i])) + 1
            assert np.array_equal(hierarchy_levels(cp, h).view(np.uint32), single[i].view(np.uint32)), (kind, i)
        big = [i for i, n in enumerate(sides) if n >= 8]
        batch = cp.CompressedShadow.create_batch([hs[i] for i in big], [(j, 0, 1) for j in range(len(big))])
        for j, i in enumerate(big):
            want = cp.CompressedShadow.create(cp.MinMaxHierarchy(maps[i])).get_dag()
            assert np.array_equal(batch[j].get_dag(), want), (kind, i)


def test_build_matches_reference(cp, golden, golden_cases):
    for key in golden_cases:
        name, zi, zn = split_key(key)
        depth = golden[f"{name}/depth"]
        nl, tv, lm = golden[f"{key}/meta"].tolist()
        mm = cp.MinMaxHierarchy(depth)
        sh = cp.CompressedShadow.create(mm, zi, zn)
        assert sh.get_num_levels() == nl and sh.uses_leafmasks() == bool(lm), key
        assert np.array_equal(sh.get_dag(), golden[f"{key}/dag"]), key
        assert sh.get_total_visibility() == tv, key
        assert np.array_equal(sh.lookup_ndc(golden[f"{name}/ndc"]), golden[f"{key}/vis"]), key


def test_reference_unit_test_traversals(cp, golden):
    """test/CompressedShadowTest.cpp:50-152 through the drop-in traverse()."""
    sh8 = cp.CompressedShadow.create(cp.MinMaxHierarchy(golden["test_depths8x8/depth"]))
    assert sh8.traverse((-1, 1, -1), False) == cp.SHADOW
    assert sh8.traverse((-1, -1, 0), False) == cp.VISIBLE
    assert sh8.traverse((1, -1, 0.99), False) == cp.VISIBLE
    sh16 = cp.CompressedShadow.create(cp.MinMaxHierarchy(golden["test_depths16x16/depth"]))
    s = 2.0 / 16.0
    assert sh16.traverse((0 + s, 0, .9)) == cp.SHADOW
    assert sh16.traverse((0 + 3 * s, 0, -.9)) == cp.VISIBLE
    sh32 = cp.CompressedShadow.create(cp.MinMaxHierarchy(golden["test_depths32x32/depth"]))
    lit = np.asarray([[x / 32.0, y / 32.0, 0.59] for y in range(31) for x in range(31)], np.float32) * 2 - 1
    assert (sh32.lookup_ndc(lit) == cp.VISIBLE).all()
    dark = np.asarray([[x / 32.0, y / 32.0, 0.79] for y in range(8, 26) for x in range(7, 27)], np.float32) * 2 - 1
    assert (sh32.lookup_ndc(dark) == cp.SHADOW).all()


# ------------------------------------------------------------- vs the oracle
def random_map(rng, n, kind):
    if kind == 0:
        return rng.random((n, n), dtype=np.float32)
    if kind == 1:
        return (rng.integers(0, 8, (n, n)) / 7).astype(np.float32)
    if kind == 2:
        return scene.rasterise(scene.make_scene(n, 0.9, int(rng.integers(1, 30)), int(rng.integers(0, 6)),
                                                int(rng.integers(1 << 30))))
    if kind == 3:
        return (rng.integers(0, 4, (n, n)) / 4).astype(np.float32)  # dyadic: SVOs that stop early
    return (rng.random((n, n)) * 0.2 + 0.7).astype(np.float32)


def check_against_oracle(cp, oracle, depth, zi=0, zn=1, leafmasks=True, nq=4096, seed=0):
    want = oracle.build(depth, zi, zn, leafmasks=leafmasks)
    sh = cp.CompressedShadow.create(cp.MinMaxHierarchy(depth), zi, zn, leafmasks=leafmasks)
    got = sh.get_dag()
    assert sh.get_num_levels() == want.num_levels
    assert sh.uses_leafmasks() == want.leafmasks
    assert got.size == want.dag.size and np.array_equal(got, want.dag)
    tree, uniq = sh.level_counts()
    assert tree == want.tree_nodes and uniq == want.unique_nodes
    n = depth.shape[0]
    rng = np.random.default_rng(seed)
    vox = rng.integers(-2, n + 2, (nq, 3)).astype(np.int32)
    assert np.array_equal(sh.lookup_voxel(vox), oracle.lookup_voxel(want.dag, want.num_levels, want.leafmasks, vox))
    ndc = rng.uniform(-1.05, 1.05, (nq, 3)).astype(np.float32)
    assert np.array_equal(sh.lookup_ndc(ndc), oracle.lookup_ndc(want.dag, want.num_levels, want.leafmasks, ndc))
    return sh


def test_random_maps_match_oracle(cp, oracle):
    rng = np.random.default_rng(1234)
    for trial in range(60):
        n = int(rng.choice([8, 16, 32, 64, 128, 256]))
        zn = int(rng.choice([1, 1, 2, 3, 5, 8]))
        check_against_oracle(cp, oracle, random_map(rng, n, trial % 5), int(rng.integers(0, zn)), zn, seed=trial)


def test_leafmasks_off_matches_oracle(cp, oracle):
    rng = np.random.default_rng(5)
    for trial in range(12):
        n = int(rng.choice([16, 32, 64, 128]))
        check_against_oracle(cp, oracle, random_map(rng, n, trial % 5), leafmasks=False, seed=trial)


def test_special_values_match_oracle(cp, oracle):
    rng = np.random.default_rng(6)
    d = (rng.random((64, 64), dtype=np.float32) * 0.6 + 0.2).astype(np.float32)
    d[rng.random((64, 64)) < 0.1] = np.float32(-0.0)
    d[rng.random((64, 64)) < 0.1] = np.float32(0.0)
    d[rng.random((64, 64)) < 0.02] = np.float32(np.nan)
    d[rng.random((64, 64)) < 0.02] = np.float32(np.inf)
    d[rng.random((64, 64)) < 0.02] = np.float32(-1.5)
    mm = cp.MinMaxHierarchy(d)
    assert np.array_equal(hierarchy_levels(cp, mm).view(np.uint32), oracle.pyramid(d).view(np.uint32))
    check_against_oracle(cp, oracle, d)
    for v in (0.0, 1.0, 0.25, 0.5, 0.3):
        check_against_oracle(cp, oracle, np.full((32, 32), v, np.float32))


def boundary_map(rng, n, H):
    """Depths whose d*H lands on or a few ulps beside voxel centres z + 0.5
    (the lit test's boundary), plus tiny, denormal and negative values."""
    z = rng.integers(-2, H + 2, (n, n))
    d = ((z + 0.5) / H).astype(np.float32)
    steps = rng.integers(-3, 4, (n, n))
    for k in range(3):
        d = np.where(steps > k, np.nextafter(d, np.float32(np.inf)), d)
        d = np.where(steps < -k, np.nextafter(d, np.float32(-np.inf)), d)
    special = np.array([0.5 / H, np.nextafter(np.float32(0.5 / H), np.float32(0)), 1e-40, -1e-40, 1e-30, -0.0,
                        0.5 - 2 ** -25, np.float32(8.5 / H), 7.5 / H], np.float32)
    pick = rng.random((n, n)) < 0.1
    d[pick] = special[rng.integers(0, special.size, int(pick.sum()))]
    return d.astype(np.float32)


def test_voxel_boundary_values_match_oracle(cp, oracle):
    rng = np.random.default_rng(77)
    for trial, (n, zn) in enumerate([(64, 1), (64, 3), (128, 8), (32, 5), (256, 1), (64, 2)]):
        zi = int(rng.integers(0, zn))
        check_against_oracle(cp, oracle, boundary_map(rng, n, n * zn), zi, zn, seed=trial)


def test_c0_config_matches_oracle(cp, oracle):
    """The 1024^2 map of 40 boxes: DAG words and 2^20 voxel lookups."""
    d = scene.rasterise(scene.config_scene("c0"))
    want = oracle.build(d)
    sh = cp.CompressedShadow.from_depth(d)
    assert np.array_equal(sh.get_dag(), want.dag)
    q = scene.voxel_queries(1 << 20, 1024, 0)
    assert np.array_equal(sh.lookup_voxel(q), oracle.lookup_voxel(want.dag, want.num_levels, True, q, threads=8))


def test_c1_config_matches_oracle(cp, oracle):
    """The 8192^2 map of 500 boxes and 64 spheres: DAG words, per-level node
    counts, and 2^22 of the mixed surface/volume NDC queries."""
    d = scene.rasterise(scene.config_scene("c1"))
    want = oracle.build(d, threads=4)
    import torch
    sh = cp.CompressedShadow.from_depth(torch.from_numpy(d).cuda())
    got = sh.get_dag()
    assert got.size == want.dag.size and np.array_equal(got, want.dag)
    tree, uniq = sh.level_counts()
    assert tree == want.tree_nodes and uniq == want.unique_nodes
    q = scene.ndc_queries_mixed(d, 1 << 22, 1)
    assert np.array_equal(sh.lookup_ndc(q), oracle.lookup_ndc(want.dag, want.num_levels, True, q, threads=8))


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_c0_config_matches_reference(cp, golden_configs):
    """The 1024^2 workload against the reference's own output
    (tests/golden/make_golden_configs.py): DAG words, per-level counts, and
    the reference's traverse answers on 2^16 mixed NDC points and on the
    voxel centres of the first 2^16 voxel queries (voxel and NDC input)."""
    g = golden_configs
    d = scene.rasterise(scene.config_scene("c0"))
    assert _sha(d) == str(g["c0/map_sha256"])
    sh = cp.CompressedShadow.from_depth(d)
    nl, tv, words = g["c0/meta"].tolist()
    assert sh.get_num_levels() == nl and sh.get_total_visibility() == tv
    assert np.array_equal(sh.get_dag(), g["c0/dag"])
    tree, uniq = sh.level_counts()
    assert tree == g["c0/tree_nodes"].tolist() and uniq == g["c0/unique_nodes"].tolist()
    q = scene.ndc_queries_mixed(d, 1 << 16, int(g["c0/ndc_seed"]))
    assert np.array_equal(sh.lookup_ndc(q), g["c0/ndc_vis"])
    v = scene.voxel_queries(1 << 20, 1024, 0)[:1 << 16]
    assert _sha(v) == str(g["c0/voxel_sha256"])
    assert np.array_equal(sh.lookup_voxel(v), g["c0/voxel_vis"])


def test_c1_config_matches_reference(cp, golden_configs):
    """The 8192^2 workload against the reference's own output: DAG length
    and SHA-256, per-level tree and unique node counts, numLevels, total
    visibility, and the reference's traverse answers on 2^16 mixed NDC
    points."""
    import torch
    g = golden_configs
    d = scene.rasterise(scene.config_scene("c1"))
    assert _sha(d) == str(g["c1/map_sha256"])
    sh = cp.CompressedShadow.from_depth(torch.from_numpy(d).cuda())
    nl, tv, words = g["c1/meta"].tolist()
    assert sh.get_num_levels() == nl and sh.get_total_visibility() == tv
    dag = sh.get_dag()
    assert dag.size == words and _sha(dag) == str(g["c1/dag_sha256"])
    tree, uniq = sh.level_counts()
    assert tree == g["c1/tree_nodes"].tolist() and uniq == g["c1/unique_nodes"].tolist()
    q = scene.ndc_queries_mixed(d, 1 << 16, int(g["c1/ndc_seed"]))
    assert np.array_equal(sh.lookup_ndc(q), g["c1/ndc_vis"])


def test_lookup_variants_agree(cp, oracle):
    """Every queries-per-thread variant of the lookup kernel (and the tuned
    choice) answers exactly like the oracle, for NDC and voxel input."""
    d = scene.rasterise(scene.config_scene("c0"))
    want = oracle.build(d)
    ctx = cp.Context(0)
    sh = cp.CompressedShadow.from_depth(d, ctx=ctx)
    q = scene.ndc_queries_mixed(d, 300_001, 9)
    v = scene.voxel_queries(200_003, 1024, 9)
    ref_q = oracle.lookup_ndc(want.dag, want.num_levels, True, q, threads=8)
    ref_v = oracle.lookup_voxel(want.dag, want.num_levels, True, v, threads=8)
    for qpt in (0, 1, 2, 4):
        ctx.set_option(ctx.OPT_LOOKUP_QUERIES_PER_THREAD, qpt)
        assert np.array_equal(sh.lookup_ndc(q), ref_q), qpt
        assert np.array_equal(sh.lookup_voxel(v), ref_v), qpt
    with pytest.raises(cp.CpvsError):
        ctx.set_option(ctx.OPT_LOOKUP_QUERIES_PER_THREAD, 3)


def test_lookup_every_depth_and_input_kind(cp, oracle):
    """Maps of sides 16..2048 put the top grid at different depths, so the
    straight-line lookup runs with 0 to several inner levels below it (and
    the looped kernel where it does not apply).  Every variant, the tuned
    choice, points in host and in device memory, and points a little
    outside [-1, 1] answer like the oracle."""
    torch = pytest.importorskip("torch")
    for n, seed in ((16, 1), (32, 2), (64, 3), (128, 4), (256, 5), (512, 6), (2048, 7)):
        d = scene.rasterise(scene.make_scene(n, 0.9, 12, 3, 600 + seed))
        want = oracle.build(d)
        ctx = cp.Context(0)
        sh = cp.CompressedShadow.from_depth(d, ctx=ctx)
        q = scene.ndc_queries_mixed(d, 20_001, seed)
        g = np.random.Generator(np.random.PCG64(seed))
        q[-2000:] = (g.random((2000, 3)) * 2.4 - 1.2).astype(np.float32)  # partly outside the volume
        ref = oracle.lookup_ndc(want.dag, want.num_levels, True, q, threads=8)
        qd = torch.from_numpy(q).cuda()
        for qpt in (0, 1, 2, 4):
            ctx.set_option(ctx.OPT_LOOKUP_QUERIES_PER_THREAD, qpt)
            assert np.array_equal(sh.lookup_ndc(q), ref), (n, qpt, "host")
            words = sh.lookup_ndc(qd).cpu().numpy().view(np.uint32)
            assert np.array_equal(cp.unpack_bits(words, q.shape[0]), ref), (n, qpt, "device")


def test_container_owns_its_shadows(cp):
    """A container takes its shadows the way the reference moves a
    unique_ptr in: a shadow stays usable while a cell holds it; one that its
    container released (container gone, cell replaced) raises on use instead
    of reaching freed memory; and a shadow cannot sit in two cells (the
    Python mirror and the C ABI both refuse)."""
    import gc
    d = scene.rasterise(scene.config_scene("c0", n=64))
    ctx = cp.Context(0)
    q = scene.ndc_queries_mixed(d, 1000, 3)
    sh = cp.CompressedShadow.from_depth(d, ctx=ctx)
    want = sh.lookup_ndc(q)
    g = cp.CompressedShadowContainer.of(sh)
    assert g.get(0, 0, 0) is sh and np.array_equal(sh.lookup_ndc(q), want)
    with pytest.raises(ValueError):
        cp.CompressedShadowContainer.of(sh)  # a cell already holds it
    other = cp.CompressedShadowContainer(2, ctx)
    with pytest.raises(ValueError):
        other.set(sh, 1, 0, 0)
    assert cp._lib.cpvs_grid_set(other.handle, 1, 0, 0, sh.handle) != 0  # the C ABI refuses too
    del g
    gc.collect()
    with pytest.raises(ValueError):
        cp.CompressedShadowContainer.of(sh)  # released with its container
    with pytest.raises(cp.CpvsError):
        sh.lookup_ndc(q)
    a = cp.CompressedShadow.from_depth(d, ctx=ctx)
    b = cp.CompressedShadow.from_depth(d, ctx=ctx)
    other.set(a, 0, 0, 0)
    other.set(b, 0, 0, 0)  # replaces (and destroys) a
    with pytest.raises(cp.CpvsError):
        a.lookup_ndc(q)
    assert np.array_equal(b.lookup_ndc(q), want)


def test_repeated_builds_are_identical(cp):
    d = scene.rasterise(scene.config_scene("c0", n=512))
    a = cp.CompressedShadow.from_depth(d).get_dag()
    for _ in range(3):
        assert np.array_equal(cp.CompressedShadow.from_depth(d).get_dag(), a)


def test_device_io_matches_host_io(cp, oracle):
    import torch
    d = scene.rasterise(scene.config_scene("c0", n=256))
    sh = cp.CompressedShadow.from_depth(torch.from_numpy(d).cuda())
    q = scene.ndc_queries_mixed(d, 100_003, 4)
    host = sh.lookup_ndc(q)
    words = sh.lookup_ndc(torch.from_numpy(q).cuda())
    torch.cuda.synchronize()
    dev = cp.unpack_bits(words.cpu().numpy().view(np.uint32), q.shape[0])
    assert np.array_equal(host, dev)
    assert sh.lookup_ndc(np.zeros((0, 3), np.float32)).size == 0


def test_grid_matches_oracle(cp, oracle):
    """A 2x2x2 grid: 2x2 xy tiles of a 128^2 map, 2 z-tiles each, plus one
    uniformly lit tile; routing and descent equal the oracle's restatement of
    shader/traverse.cs."""
    n, L = 64, 2
    full = scene.rasterise(scene.make_scene(n * L, 0.9, 20, 4, 77))
    full[:n, n:] = np.float32(1.0)  # tile (x=1, y=0) lit everywhere
    grid = cp.CompressedShadowContainer(L)
    dags, offs, off = [], [], 0
    for z in range(L):
        for y in range(L):
            for x in range(L):
                tile = np.ascontiguousarray(full[y * n:(y + 1) * n, x * n:(x + 1) * n])
                b = oracle.build(tile, z, L)
                dags.append(b.dag)
                offs.append(off)
                off += b.dag.size
                grid.set(cp.CompressedShadow.from_depth(tile, z, L), x, y, z)
    grid.copy_to_gpu()
    dag, cells = grid.words()
    assert np.array_equal(dag, np.concatenate(dags))
    q = np.random.default_rng(3).uniform(-1.1, 1.1, (200_000, 3)).astype(np.float32)
    want = oracle.grid_lookup_ndc(np.concatenate(dags).astype(np.uint32), np.asarray(offs, np.uint32), L,
                                  int(np.log2(n)) + 1, True, q)
    assert np.array_equal(grid.lookup_ndc(q), want)
    lit_cells = [(z * L + 0) * L + 1 for z in range(L)]
    assert any(cells[c] == 0xFFFFFFFE for c in lit_cells)


def test_errors(cp):
    d = scene.rasterise(scene.config_scene("c0", n=256))
    with pytest.raises(cp.CpvsError) as e:
        cp.CompressedShadow.from_depth(np.zeros((48, 48), np.float32))
    assert e.value.status == 1
    with pytest.raises(cp.CpvsError) as e:
        cp.CompressedShadow.from_depth(d, 3, 2)
    assert e.value.status == 1
    ctx = cp.Context(0)
    ctx.set_budget(1 << 20)
    with pytest.raises(cp.CpvsError) as e:
        cp.CompressedShadow.from_depth(d, ctx=ctx)
    assert e.value.status == 6
    ctx.set_budget(0)
    assert cp.CompressedShadow.from_depth(d, ctx=ctx).dag_size() > 0


# ------------------------------------------------------------ batched forms
def test_batch_matches_single_builds(cp, oracle):
    """Independent lights of uneven sizes plus z-tiles of one map, built in one
    batch (including an 8x8 map, which cannot use leafmasks): every DAG equals
    its own single build and the oracle's."""
    rng = np.random.default_rng(21)
    maps = [scene.rasterise(scene.make_scene(int(n), 0.9, int(rng.integers(5, 60)), 2, 100 + i))
            for i, n in enumerate([64, 1024, 256, 8, 512, 128, 2048, 256])]
    hs = [cp.MinMaxHierarchy(m) for m in maps]
    jobs = [(i, 0, 1) for i in range(len(maps))] + [(2, z, 4) for z in range(4)] + [(6, 1, 3)]
    batch = cp.CompressedShadow.create_batch(hs, jobs)
    q = np.random.default_rng(5).uniform(-1, 1, (50_000, 3)).astype(np.float32)
    for (src, zi, zn), sh in zip(jobs, batch):
        want = oracle.build(maps[src], zi, zn)
        single = cp.CompressedShadow.create(hs[src], zi, zn)
        assert np.array_equal(sh.get_dag(), single.get_dag()), (src, zi, zn)
        assert np.array_equal(sh.get_dag(), want.dag), (src, zi, zn)
        assert sh.level_counts() == single.level_counts()
        assert sh.get_total_visibility() == single.get_total_visibility()
        assert np.array_equal(sh.lookup_ndc(q), oracle.lookup_ndc(want.dag, want.num_levels, want.leafmasks, q))
    del batch  # handles share one device block; dropping them frees it


def test_grid_build_matches_oracle(cp, oracle):
    """cpvs_grid_build: 4x4 xy tiles of a 256^2 map, 4 z-tiles each (64
    DAGs in one batch) against per-cell oracle builds and the oracle's grid
    routing."""
    n, L = 64, 4
    full = scene.rasterise(scene.make_scene(n * L, 0.95, 60, 8, 55))
    full[:n, :n] = np.float32(1.0)  # a lit tile: uniform cells
    tiles = [np.ascontiguousarray(full[y * n:(y + 1) * n, x * n:(x + 1) * n]) for y in range(L) for x in range(L)]
    grid = cp.CompressedShadowContainer(L)
    grid.build([cp.MinMaxHierarchy(t) for t in tiles])
    dag, cells = grid.words()
    dags, offs, off = [], [], 0
    for z in range(L):
        for y in range(L):
            for x in range(L):
                b = oracle.build(tiles[y * L + x], z, L)
                dags.append(b.dag)
                offs.append(off)
                off += b.dag.size
    assert np.array_equal(dag, np.concatenate(dags))
    uniform = [i for i in range(L ** 3) if dags[i].size == 1]
    assert uniform and all(cells[i] in (0xFFFFFFFE, 0xFFFFFFFF) for i in uniform)
    q = np.random.default_rng(4).uniform(-1.05, 1.05, (300_000, 3)).astype(np.float32)
    want = oracle.grid_lookup_ndc(np.concatenate(dags).astype(np.uint32), np.asarray(offs, np.uint32), L,
                                  int(np.log2(n)) + 1, True, q)
    assert np.array_equal(grid.lookup_ndc(q), want)


def test_raster_matches_host_rasteriser(cp):
    """The CUDA depth producer equals the host rasteriser bit for bit, for
    whole maps and windows, boxes and spheres."""
    for n, nb, ns, seed in ((64, 10, 4, 1), (512, 120, 30, 2), (1024, 40, 0, 0), (2048, 500, 64, 3)):
        sc = scene.make_scene(n, 0.95, nb, ns, seed)
        want = scene.rasterise(sc)
        got = cp.raster_depth(sc).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), n
    sc = scene.make_scene(1024, 0.9, 200, 40, 7)
    full = scene.rasterise(sc)
    for x0, y0, w, h in ((0, 0, 256, 256), (256, 512, 256, 128), (1000, 3, 24, 100)):
        got = cp.raster_depth(sc, x0, y0, w, h).cpu().numpy()
        assert np.array_equal(got, full[y0:y0 + h, x0:x0 + w]), (x0, y0, w, h)


def test_multi_dag_lookup_matches_single_lookups(cp, oracle):
    """Queries spread over many resident DAGs in one launch answer exactly as
    each DAG's own lookup (and the oracle)."""
    import torch
    rng = np.random.default_rng(31)
    sizes = [64, 256, 1024, 128, 512, 16, 2048, 256]
    maps = [scene.rasterise(scene.make_scene(n, 0.9, 30, 3, 300 + i)) for i, n in enumerate(sizes)]
    hs = [cp.MinMaxHierarchy(m) for m in maps]
    shadows = cp.CompressedShadow.create_batch(hs, [(i, 0, 1) for i in range(len(maps))])
    nq = 400_000
    ids = rng.integers(0, len(maps) + 1, nq).astype(np.uint32)  # the last id is outside the table
    q = rng.uniform(-1, 1, (nq, 3)).astype(np.float32)
    got = cp.lookup_ndc_multi(shadows, ids, q)
    for i, sh in enumerate(shadows):
        sel = ids == i
        assert np.array_equal(got[sel], sh.lookup_ndc(q[sel])), i
    assert (got[ids == len(maps)] == 0).all()
    dev = cp.lookup_ndc_multi(shadows, torch.from_numpy(ids).cuda(), torch.from_numpy(q).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(cp.unpack_bits(dev.cpu().numpy().view(np.uint32), nq), got)


def test_host_map_may_be_reused_on_return(cp, oracle):
    """cpvs_hierarchy_create reads a host map in place where the GPU can: the
    call returns only when the map has been read, so the caller may overwrite
    or free it right away (here: overwritten immediately, many times)."""
    rng = np.random.default_rng(21)
    maps = [random_map(rng, 64, k % 5) for k in range(12)]
    buf = np.empty((64, 64), np.float32)
    for k, m in enumerate(maps):
        buf[:] = m
        mm = cp.MinMaxHierarchy(buf)
        buf[:] = np.float32(np.nan)  # clobber the caller's buffer after the call
        got = cp.CompressedShadow.create(mm).get_dag()
        assert np.array_equal(got, oracle.build(m).dag), k


def test_plan_grows_for_a_busier_map(cp, oracle):
    """A plan sized by a nearly flat map overflows on a noisy map of the same
    side: the build re-plans from the new map's level bounds and retries, and
    every DAG still equals the oracle's (then the grown plan serves both)."""
    ctx = cp.Context(0)
    flat = np.full((512, 512), np.float32(0.9))
    flat[100:140, 200:260] = np.float32(0.4)
    noisy = np.random.default_rng(8).random((512, 512), dtype=np.float32)
    for d in (flat, noisy, flat, noisy):
        sh = cp.CompressedShadow.create(cp.MinMaxHierarchy(d, ctx=ctx))
        want = oracle.build(d)
        assert np.array_equal(sh.get_dag(), want.dag)
        assert sh.level_counts() == (want.tree_nodes, want.unique_nodes)


def test_every_build_shape_gives_the_oracles_dag(cp, oracle):
    """The build tuner times every (cluster cap, insert waves) pair on a
    plan's first build; each pair, fixed through the context options, must
    build the same DAG (the oracle's) on maps whose level sizes fall on both
    sides of every cap, including the 8192^2 workload."""
    import torch
    rng = np.random.default_rng(21)
    maps = [scene.rasterise(scene.config_scene("c0")), random_map(rng, 256, 0),
            scene.rasterise(scene.make_scene(2048, 0.9, 80, 8, 9)), scene.rasterise(scene.config_scene("c1"))]
    wants = [oracle.build(d, threads=4).dag for d in maps]
    devs = [torch.from_numpy(d).cuda() for d in maps]
    for cap in (2048, 4096, 8192, 16384):
        for waves in (1, 2):
            ctx = cp.Context(0)
            ctx.set_option(ctx.OPT_BUILD_CLUSTER_CAP, cap)
            ctx.set_option(ctx.OPT_BUILD_INSERT_WAVES, waves)
            for d, want in zip(devs, wants):
                sh = cp.CompressedShadow.from_depth(d, ctx=ctx)
                assert np.array_equal(sh.get_dag(), want), (cap, waves, d.shape)
                rep = ctx.last_build()
                assert rep["error_word"] == 0 and rep["tuned"] == 0
                assert rep["cluster_cap"] == cap and rep["insert_waves"] == waves


def test_build_tuner_times_once_per_plan(cp, oracle):
    """A fresh context's first build of a shape times the candidates and
    keeps one; the next build of that shape reuses it; both DAGs equal the
    oracle's."""
    d = scene.rasterise(scene.config_scene("c0"))
    want = oracle.build(d).dag
    ctx = cp.Context(0)
    sh = cp.CompressedShadow.from_depth(d, ctx=ctx)
    first = ctx.last_build()
    assert first["tuned"] == 1 and first["tuning_ms"] > 0 and first["error_word"] == 0
    assert first["cluster_cap"] in (2048, 4096, 8192, 16384) and first["insert_waves"] in (1, 2)
    assert np.array_equal(sh.get_dag(), want)
    sh = cp.CompressedShadow.from_depth(d, ctx=ctx)
    again = ctx.last_build()
    assert again["tuned"] == 0
    assert (again["cluster_cap"], again["insert_waves"]) == (first["cluster_cap"], first["insert_waves"])
    assert np.array_equal(sh.get_dag(), want)
