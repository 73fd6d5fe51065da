"""The header-only C++ classes (include/cpvs.hpp) that mirror the reference's
CompressedShadow / MinMaxHierarchy / CompressedShadowContainer: they compile
warning-free against the C ABI, and a program using them like the
reference's own call sites answers exactly as the oracle does."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cpvs_gb300 import scene
from oracle.oracle import split_pyramid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "cpvs_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "wrapper_demo.cpp")
BATCH_SRC = os.path.join(ROOT, "tests", "cpp", "batch_demo.cpp")


def compile_demo(out, extra=(), src=SRC):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    if not os.path.exists(os.path.join(LIBDIR, "libcpvs_gb300.so")):
        pytest.skip("library not built")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), *extra,
           src, "-L", LIBDIR, "-lcpvs_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_wrapper_compiles(tmp_path):
    compile_demo(str(tmp_path / "demo"))


def test_batch_demo_compiles(tmp_path):
    compile_demo(str(tmp_path / "batch_demo"), src=BATCH_SRC)


def test_wrapper_compiles_without_global_names(tmp_path):
    # the demo uses the global names, so only the header is checked here
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / "t.cpp"
    src.write_text('#include "cpvs.hpp"\nint main() { cpvs::vec3 v(1, 2, 3); return (int)v.x - 1; }\n'
                   "#ifdef CompressedShadow\n#error\n#endif\n")
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-DCPVS_NO_GLOBAL_NAMES", "-I",
                    os.path.join(ROOT, "include"), "-fsyntax-only", str(src)], check=True)


@pytest.mark.gpu
def test_wrapper_answers_like_the_oracle(tmp_path, oracle):
    exe = str(tmp_path / "demo")
    compile_demo(exe)
    n = 256
    depth = scene.rasterise(scene.make_scene(n, 0.9, 40, 4, 21))
    pts = np.random.default_rng(4).uniform(-1, 1, (3000, 3)).astype(np.float32)
    w, h = 40, 30
    pos = np.random.default_rng(5).uniform(-1.1, 1.1, (h, w, 4)).astype(np.float32)
    M = np.eye(4, dtype=np.float32)
    M[0, 1] = np.float32(0.1)  # a shear, so the transform is not the identity
    colmajor = np.ascontiguousarray(M.T.ravel(), np.float32)
    for name, arr in (("depth", depth), ("pts", pts), ("pos", pos), ("m", colmajor)):
        arr.astype(np.float32).tofile(tmp_path / f"{name}.f32")
    out = str(tmp_path / "out")
    r = subprocess.run([exe, str(n), str(tmp_path / "depth.f32"), str(len(pts)), str(tmp_path / "pts.f32"), str(w),
                        str(h), str(tmp_path / "pos.f32"), str(tmp_path / "m.f32"), "3", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    b = oracle.build(depth)
    assert np.array_equal(np.fromfile(out + ".dag", np.uint32), b.dag)
    nl, total, mm_levels, mn, mx, d01 = open(out + ".meta").read().split()
    assert int(nl) == b.num_levels == int(mm_levels)
    level1 = split_pyramid(oracle.pyramid(depth), n)[0]
    assert np.float32(mn) == level1[0, 0, 0] and np.float32(mx) == level1[0, 0, 1]
    assert np.float32(d01) == depth[0, 1]  # getMin(0, x=1, y=0) is the map itself
    want = oracle.lookup_ndc(b.dag, b.num_levels, True, pts)
    assert np.array_equal(np.fromfile(out + ".trav", np.uint8), want)
    want_eval = oracle.grid_evaluate(b.dag, np.zeros(1, np.uint32), 1, b.num_levels, True, pos, colmajor, 3)
    assert np.array_equal(np.fromfile(out + ".eval", np.uint8).reshape(h, w), want_eval)


@pytest.mark.gpu
def test_batch_classes_answer_like_the_oracle(tmp_path, oracle):
    """MinMaxHierarchy::createBatch, CompressedShadow::createBatch and
    CompressedShadowContainer::build: every DAG equals the oracle's."""
    exe = str(tmp_path / "batch_demo")
    compile_demo(exe, src=BATCH_SRC)
    sides = [64, 128, 8, 256]
    maps = [scene.rasterise(scene.make_scene(n, 0.9, 20 + i, 3, 70 + i)) for i, n in enumerate(sides)]
    np.concatenate([m.ravel() for m in maps]).astype(np.float32).tofile(tmp_path / "maps.f32")
    n, L = 64, 2
    full = scene.rasterise(scene.make_scene(n * L, 0.95, 30, 4, 77))
    full[:n, :n] = np.float32(1.0)  # a lit tile: uniform cells
    tiles = [np.ascontiguousarray(full[y * n:(y + 1) * n, x * n:(x + 1) * n]) for y in range(L) for x in range(L)]
    np.concatenate([t.ravel() for t in tiles]).astype(np.float32).tofile(tmp_path / "tiles.f32")
    out = str(tmp_path / "out")
    r = subprocess.run([exe, str(len(sides)), *map(str, sides), str(tmp_path / "maps.f32"), str(L), str(n),
                        str(tmp_path / "tiles.f32"), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    hier, flags = open(out + ".meta").read().split("\n")[:2]
    hier = hier.split()
    for i, m in enumerate(maps):
        level1 = split_pyramid(oracle.pyramid(m), sides[i])[0]
        assert int(hier[3 * i]) == int(np.log2(sides[i])) + 1
        assert np.float32(hier[3 * i + 1]) == level1[0, 0, 0] and np.float32(hier[3 * i + 2]) == level1[0, 0, 1]
    jobs = [(i, 0, 1) for i in range(len(sides))] + [(0, 1, 2)]
    for j, (src, zi, zn) in enumerate(jobs):
        want = oracle.build(maps[src], zi, zn)
        assert np.array_equal(np.fromfile(f"{out}.dag{j}", np.uint32), want.dag), (src, zi, zn)
    assert flags.split() == ["1", "1", "1"]  # cells released, wrong tile count refused, grid kept
    dags, offs, off = [], [], 0
    for z in range(L):
        for y in range(L):
            for x in range(L):
                b = oracle.build(tiles[y * L + x], z, L)
                dags.append(b.dag)
                offs.append(off)
                off += b.dag.size
    assert np.array_equal(np.fromfile(out + ".grid", np.uint32), np.concatenate(dags))
    cells = np.fromfile(out + ".cells", np.uint32)
    for i, d in enumerate(dags):
        assert cells[i] in (0xFFFFFFFE, 0xFFFFFFFF) if d.size == 1 else cells[i] == offs[i], i
