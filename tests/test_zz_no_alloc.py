"""The allocation-free build, cpvs_shadow_build_noalloc, called through the C
ABI.  It serves callers that may not allocate device memory (a render loop
that must not stall on cudaMalloc/cudaFree, a plugin inside an application
that owns all GPU memory): its scratch is a fixed array inside the library.
Its DAG must equal the one the allocating build makes and the oracle's,
call after call, although every call reuses the same array.  This file is
collected last so that a run stopping at the first failure has run
everything else first."""
import ctypes as C

import numpy as np
import pytest

from cpvs_gb300 import scene

pytestmark = pytest.mark.gpu


def build_noalloc(lib, depth_dev, n, capacity, z_index=0, z_num=1, leafmasks=True):
    import torch
    out = torch.zeros(max(capacity, 1), dtype=torch.int32, device=depth_dev.device)
    words = C.c_uint64(0)
    status = lib.cpvs_shadow_build_noalloc(depth_dev.data_ptr(), n, z_index, z_num, 1 if leafmasks else 0,
                                           out.data_ptr(), capacity, C.byref(words), None)
    return status, out[:words.value].cpu().numpy().view(np.uint32), words.value


def test_noalloc_matches_allocating_build(cp):
    import torch
    lib = cp.load_library()
    maps = [scene.rasterise(scene.make_scene(256, 0.9, 30, 4, 41)),
            scene.rasterise(scene.make_scene(64, 0.95, 10, 2, 42)),
            scene.rasterise(scene.make_scene(256, 0.9, 30, 4, 41))]
    for depth, (zi, zn) in zip(maps, [(0, 1), (1, 3), (0, 1)]):   # calls in a row share the scratch
        n = depth.shape[0]
        want = cp.CompressedShadow.from_depth(depth, zi, zn).get_dag()
        d = torch.from_numpy(depth).cuda()
        status, got, words = build_noalloc(lib, d, n, 1 << 20, zi, zn)
        assert status == 0, lib.cpvs_last_error()
        assert words == want.size
        assert np.array_equal(got, want)


def test_noalloc_without_leafmasks_and_small_maps(cp):
    import torch
    lib = cp.load_library()
    rng = np.random.default_rng(8)
    for n, leaf in ((8, True), (16, False), (32, False)):
        depth = (rng.random((n, n)) * 0.5 + 0.3).astype(np.float32)
        want = cp.CompressedShadow.from_depth(depth, leafmasks=leaf).get_dag()
        status, got, _ = build_noalloc(lib, torch.from_numpy(depth).cuda(), n, 1 << 16, leafmasks=leaf)
        assert status == 0, lib.cpvs_last_error()
        assert np.array_equal(got, want)


def test_noalloc_matches_oracle(cp, oracle):
    """Random maps of five kinds and maps whose depths sit on or beside voxel
    boundaries, with and without z-tiles, against the oracle's DAG words
    (the multi-pass kernels the allocation-free build runs are used by no
    other path)."""
    import torch
    from test_gpu_parity import boundary_map, random_map
    lib = cp.load_library()
    rng = np.random.default_rng(4321)
    cases = [(random_map(rng, int(rng.choice([16, 32, 64, 128, 256])), kind), kind)
             for kind in range(5) for _ in range(3)]
    for n, zn in ((64, 1), (64, 3), (128, 8), (256, 1), (32, 5)):
        cases.append((boundary_map(rng, n, n * zn), zn))
    for t, (depth, zk) in enumerate(cases):
        n = depth.shape[0]
        zn = zk if t >= 15 else int(rng.choice([1, 1, 2, 3]))
        zi = int(rng.integers(0, zn))
        want = oracle.build(depth, zi, zn)
        status, got, words = build_noalloc(lib, torch.from_numpy(depth).cuda(), n, 1 << 22, zi, zn)
        assert status == 0, lib.cpvs_last_error()
        assert words == want.dag.size and np.array_equal(got, want.dag), (t, n, zi, zn)
    for n in (16, 32, 64):
        depth = random_map(rng, n, 2)
        want = oracle.build(depth, leafmasks=False)
        status, got, _ = build_noalloc(lib, torch.from_numpy(depth).cuda(), n, 1 << 22, leafmasks=False)
        assert status == 0 and np.array_equal(got, want.dag), n


def test_noalloc_limits(cp):
    import torch
    lib = cp.load_library()
    big = torch.zeros((512, 512), dtype=torch.float32, device="cuda")
    status, _, _ = build_noalloc(lib, big, 512, 1 << 16)
    assert status == 1 and b"256" in lib.cpvs_last_error()      # beyond the fixed maximum
    small = torch.zeros((128, 128), dtype=torch.float32, device="cuda")
    status, _, _ = build_noalloc(lib, small, 128, 1 << 16, leafmasks=False)
    assert status == 1 and b"64" in lib.cpvs_last_error()       # without leafmasks: at most 64
    words = C.c_uint64(0)
    out = torch.zeros(1 << 16, dtype=torch.int32, device="cuda")
    status = lib.cpvs_shadow_build_noalloc(small.data_ptr(), 128, 0, 1, 0x1 | 0x100, out.data_ptr(), 1 << 16,
                                           C.byref(words), None)
    assert status == 1 and b"flag" in lib.cpvs_last_error()     # unknown flag bits
    depth = torch.from_numpy(scene.rasterise(scene.make_scene(128, 0.9, 20, 2, 5))).cuda()
    status, _, words = build_noalloc(lib, depth, 128, 4)
    assert status == 8 and words > 4                             # output too small: size reported
    status, got, _ = build_noalloc(lib, depth, 128, words)
    assert status == 0 and got.size == words
