"""Saved DAGs (cpvs_shadow_serialize / cpvs_grid_serialize and their
loaders): the C implementation writes exactly the bytes the numpy
description (cpvs_gb300/dagfile.py) defines, loads files produced from the
oracle's DAGs, round-trips shadows and grids, and rejects damaged files."""
import numpy as np
import pytest

from cpvs_gb300 import dagfile, scene


def test_fnv1a64_known_answers():
    # published FNV-1a 64 test vectors
    assert dagfile.fnv1a64(b"") == 0xCBF29CE484222325
    assert dagfile.fnv1a64(b"a") == 0xAF63DC4C8601EC8C
    assert dagfile.fnv1a64(b"foobar") == 0x85944171F73967E8


def test_pack_unpack_oracle_dag(oracle):
    d = scene.rasterise(scene.make_scene(128, 0.9, 20, 2, 5))
    b = oracle.build(d)
    blob = dagfile.pack_shadow(b.dag, b.num_levels, b.leafmasks, b.tree_nodes, b.unique_nodes)
    assert blob[:8] == b"CPVSDAG\0" and len(blob) == 48 + 16 * b.num_levels + 4 * b.dag.size
    u = dagfile.unpack(blob)
    assert np.array_equal(u["dag"], b.dag) and u["num_levels"] == b.num_levels and u["leafmasks"]
    assert u["tree_nodes"] == b.tree_nodes and u["unique_nodes"] == b.unique_nodes
    bad = bytearray(blob)
    bad[100] ^= 1
    with pytest.raises(ValueError):
        dagfile.unpack(bytes(bad))
    with pytest.raises(ValueError):
        dagfile.unpack(blob[:-4])


@pytest.mark.gpu
def test_shadow_bytes_equal_the_format_of_the_oracle_dag(cp, oracle, tmp_path):
    d = scene.rasterise(scene.make_scene(512, 0.9, 40, 4, 6))
    b = oracle.build(d)
    sh = cp.CompressedShadow.from_depth(d)
    blob = sh.to_bytes()
    assert blob == dagfile.pack_shadow(b.dag, b.num_levels, b.leafmasks, b.tree_nodes, b.unique_nodes)
    # a file made without the GPU loads and answers like the oracle
    path = tmp_path / "s.cpvs"
    path.write_bytes(dagfile.pack_shadow(b.dag, b.num_levels, b.leafmasks, b.tree_nodes, b.unique_nodes))
    loaded = cp.CompressedShadow.load(str(path))
    assert np.array_equal(loaded.get_dag(), b.dag)
    assert loaded.level_counts() == (b.tree_nodes, b.unique_nodes)
    q = np.random.default_rng(1).uniform(-1, 1, (100_000, 3)).astype(np.float32)
    assert np.array_equal(loaded.lookup_ndc(q), oracle.lookup_ndc(b.dag, b.num_levels, True, q))
    assert loaded.get_total_visibility() == sh.get_total_visibility()


@pytest.mark.gpu
def test_grid_round_trip_and_damaged_files(cp):
    n, L = 128, 2
    full = scene.rasterise(scene.make_scene(n * L, 0.9, 30, 4, 8))
    grid = cp.CompressedShadowContainer(L)
    for z in range(L):
        for y in range(L):
            for x in range(L):
                tile = np.ascontiguousarray(full[y * n:(y + 1) * n, x * n:(x + 1) * n])
                grid.set(cp.CompressedShadow.from_depth(tile, z, L), x, y, z)
    grid.copy_to_gpu()
    blob = grid.to_bytes()
    dag, cells = grid.words()
    assert blob == dagfile.pack_grid(dag, cells, L, int(np.log2(n)) + 1, True)
    g2 = cp.CompressedShadowContainer.from_bytes(blob)
    d2, c2 = g2.words()
    assert np.array_equal(d2, dag) and np.array_equal(c2, cells)
    q = np.random.default_rng(2).uniform(-1.05, 1.05, (200_000, 3)).astype(np.float32)
    assert np.array_equal(g2.lookup_ndc(q), grid.lookup_ndc(q))
    pos = np.random.default_rng(3).uniform(-1, 1, (64, 80, 4)).astype(np.float32)
    assert np.array_equal(g2.evaluate(pos, np.eye(4)), grid.evaluate(pos, np.eye(4)))
    for bad in (blob[:-1], blob[:40], b"X" + blob[1:], blob[:60] + bytes([blob[60] ^ 0x10]) + blob[61:]):
        with pytest.raises(cp.CpvsError) as e:
            cp.CompressedShadowContainer.from_bytes(bad)
        assert e.value.status == 1
    with pytest.raises(cp.CpvsError):
        cp.CompressedShadow.from_bytes(blob)  # a grid is not a shadow
    # a cell offset outside the DAG is refused even with a valid checksum
    cells_bad = cells.copy()
    cells_bad[0] = dag.size + 5
    with pytest.raises(cp.CpvsError):
        cp.CompressedShadowContainer.from_bytes(dagfile.pack_grid(dag, cells_bad, L, int(np.log2(n)) + 1, True))
