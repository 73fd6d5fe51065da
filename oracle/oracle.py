"""ctypes bindings for the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product.

* ``Oracle`` wraps liboracle.so, the C++ restatement in cpvs_oracle.cpp.
* ``Reference`` wraps _ref/libcpvs_ref.so, the reference's own sources
  compiled in place (only buildable where the reference checkout exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcpvs_ref.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

SHADOW, VISIBLE, PARTIAL = 0, 1, 2
FLAG_LEAFMASKS, FLAG_LINEAR_MERGE = 1, 2


def build_oracle(ref_dir: str | None = None) -> None:
    """Compile liboracle.so (and, when the reference checkout exists, the
    reference build under _ref/)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref_dir and os.path.isdir(ref_dir):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True)


def pyramid_floats(n: int) -> int:
    tot, s = 0, n >> 1
    while s >= 1:
        tot += 2 * s * s
        s >>= 1
    return tot


def split_pyramid(flat: np.ndarray, n: int) -> list:
    """Flat levels 1..log2(n) -> list of (s, s, 2) arrays (index 0 = level 1)."""
    out, o, s = [], 0, n >> 1
    while s >= 1:
        out.append(flat[o:o + 2 * s * s].reshape(s, s, 2))
        o += 2 * s * s
        s >>= 1
    return out


class _Built:
    def __init__(self, dag: np.ndarray, num_levels: int, leafmasks: bool, ref_defined: bool = True,
                 tree_nodes=None, unique_nodes=None):
        self.dag = dag
        self.num_levels = num_levels
        self.leafmasks = leafmasks
        self.ref_defined = ref_defined
        self.tree_nodes = tree_nodes or []
        self.unique_nodes = unique_nodes or []


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(
                os.path.join(HERE, "cpvs_oracle.cpp")):
            build_oracle()
        L = C.CDLL(path)
        L.oracle_pyramid.argtypes = [_f32p, C.c_uint32, _f32p, C.c_int]
        L.oracle_pyramid.restype = C.c_int
        L.oracle_child_mask.argtypes = [_f32p, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32]
        L.oracle_child_mask.restype = C.c_uint32
        L.oracle_build.argtypes = [_f32p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]
        L.oracle_build.restype = C.c_void_p
        for name, rt in (("oracle_dag_size", C.c_size_t), ("oracle_num_levels", C.c_uint32),
                         ("oracle_uses_leafmasks", C.c_int), ("oracle_ref_defined", C.c_int)):
            getattr(L, name).argtypes = [C.c_void_p]
            getattr(L, name).restype = rt
        L.oracle_dag_words.argtypes = [C.c_void_p]
        L.oracle_dag_words.restype = C.POINTER(C.c_uint32)
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_tree_nodes.argtypes = [C.c_void_p, C.c_int]
        L.oracle_tree_nodes.restype = C.c_uint64
        L.oracle_unique_nodes.argtypes = [C.c_void_p, C.c_int]
        L.oracle_unique_nodes.restype = C.c_uint64
        L.oracle_total_visibility.argtypes = [_u32p]
        L.oracle_total_visibility.restype = C.c_int
        L.oracle_lookup_voxel.argtypes = [_u32p, C.c_uint32, C.c_int, _i32p, C.c_uint64, _u8p, C.c_int]
        L.oracle_lookup_ndc.argtypes = [_u32p, C.c_uint32, C.c_int, _f32p, C.c_uint64, _u8p, C.c_int]
        L.oracle_grid_lookup_ndc.argtypes = [_u32p, _u32p, C.c_uint32, C.c_uint32, C.c_int, _f32p,
                                             C.c_uint64, _u8p, C.c_int]
        L.oracle_grid_evaluate.argtypes = [_u32p, _u32p, C.c_uint32, C.c_uint32, C.c_int, _f32p, C.c_uint64,
                                           C.c_uint32, _f32p, C.c_uint32, _u8p, C.c_int]
        L.oracle_shade.argtypes = [C.c_uint64, _f32p, C.c_uint32, _f32p, C.c_void_p, C.c_void_p, C.c_uint32,
                                   C.c_void_p, C.c_uint32, C.c_void_p, _f32p, _f32p]
        L.oracle_merge_level.argtypes = [_u32p, C.c_uint32, C.c_uint32, _u32p, _u32p]
        L.oracle_merge_level.restype = C.c_uint32
        self.lib = L

    def merge_level(self, words, node_size):
        w = np.ascontiguousarray(words, np.uint32)
        out = np.zeros_like(w)
        mapping = np.zeros(w.size // node_size, np.uint32)
        left = self.lib.oracle_merge_level(w, w.size, node_size, out, mapping)
        return out, mapping, int(left)

    def pyramid(self, depth: np.ndarray, threads: int = 1) -> np.ndarray:
        d = np.ascontiguousarray(depth, np.float32)
        n = d.shape[0]
        out = np.zeros(pyramid_floats(n), np.float32)
        self.lib.oracle_pyramid(d.reshape(-1), n, out, threads)
        return out

    def child_mask(self, depth, level, x, y, z, z_num=1) -> int:
        d = np.ascontiguousarray(depth, np.float32)
        return int(self.lib.oracle_child_mask(d.reshape(-1), d.shape[0], level, x, y, z, z_num))

    def build(self, depth: np.ndarray, z_index: int = 0, z_num: int = 1, leafmasks: bool = True,
              linear_merge: bool = False, threads: int = 1) -> _Built:
        d = np.ascontiguousarray(depth, np.float32)
        n = d.shape[0]
        flags = (FLAG_LEAFMASKS if leafmasks else 0) | (FLAG_LINEAR_MERGE if linear_merge else 0)
        h = self.lib.oracle_build(d.reshape(-1), n, z_index, z_num, flags, threads)
        try:
            size = self.lib.oracle_dag_size(h)
            dag = np.ctypeslib.as_array(self.lib.oracle_dag_words(h), shape=(size,)).copy() if size else \
                np.zeros(0, np.uint32)
            nl = int(self.lib.oracle_num_levels(h))
            res = _Built(dag.astype(np.uint32), nl, bool(self.lib.oracle_uses_leafmasks(h)),
                         bool(self.lib.oracle_ref_defined(h)),
                         [int(self.lib.oracle_tree_nodes(h, L)) for L in range(nl)],
                         [int(self.lib.oracle_unique_nodes(h, L)) for L in range(nl)])
        finally:
            self.lib.oracle_free(h)
        return res

    def lookup_voxel(self, dag, num_levels, leafmasks, xyz, threads: int = 1) -> np.ndarray:
        q = np.ascontiguousarray(xyz, np.int32).reshape(-1)
        out = np.zeros(q.size // 3, np.uint8)
        self.lib.oracle_lookup_voxel(np.ascontiguousarray(dag, np.uint32), num_levels, int(leafmasks), q,
                                     out.size, out, threads)
        return out

    def lookup_ndc(self, dag, num_levels, leafmasks, xyz, threads: int = 1) -> np.ndarray:
        q = np.ascontiguousarray(xyz, np.float32).reshape(-1)
        out = np.zeros(q.size // 3, np.uint8)
        self.lib.oracle_lookup_ndc(np.ascontiguousarray(dag, np.uint32), num_levels, int(leafmasks), q,
                                   out.size, out, threads)
        return out

    def grid_evaluate(self, dag, cell_offsets, length, dag_levels, leafmasks, positions, light_view_proj_colmajor,
                      filter_size: int = 1, threads: int = 1):
        """(H, W) uint8 visibilities of an (H, W, C>=3) position image."""
        h, w, fpp = positions.shape
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        m = np.ascontiguousarray(light_view_proj_colmajor, np.float32).reshape(16)
        out = np.zeros(h * w, np.uint8)
        self.lib.oracle_grid_evaluate(np.ascontiguousarray(dag, np.uint32),
                                      np.ascontiguousarray(cell_offsets, np.uint32), length, dag_levels,
                                      int(leafmasks), pos, h * w, fpp, m, filter_size, out, threads)
        return out.reshape(h, w)

    def shade(self, normals, albedo, light_direction, visibilities=None, positions=None, shadow_map=None,
              light_view_proj_colmajor=None):
        """(H, W, 4) float32 colours of the shading pass: (H, W, C>=3) normals,
        (H, W, 4) albedo, and either (H, W) uint8 visibilities or the
        shadow-map test on (H, W, C>=3) positions against a square depth map."""
        h, w, fpn = normals.shape
        nrm = np.ascontiguousarray(normals, np.float32).reshape(-1)
        alb = np.ascontiguousarray(albedo, np.float32).reshape(-1)
        light = np.ascontiguousarray(light_direction, np.float32).reshape(3)
        out = np.zeros((h, w, 4), np.float32)
        if visibilities is not None:
            vis = np.ascontiguousarray(visibilities, np.uint8).reshape(-1)
            self.lib.oracle_shade(h * w, nrm, fpn, alb, vis.ctypes.data, None, 0, None, 0, None, light, out.reshape(-1))
        else:
            pos = np.ascontiguousarray(positions, np.float32)
            sm = np.ascontiguousarray(shadow_map, np.float32)
            m = np.ascontiguousarray(light_view_proj_colmajor, np.float32).reshape(16)
            self.lib.oracle_shade(h * w, nrm, fpn, alb, None, pos.ctypes.data, pos.shape[-1], sm.ctypes.data,
                                  sm.shape[0], m.ctypes.data, light, out.reshape(-1))
        return out

    def grid_lookup_ndc(self, dag, cell_offsets, length, dag_levels, leafmasks, xyz, threads: int = 1):
        q = np.ascontiguousarray(xyz, np.float32).reshape(-1)
        out = np.zeros(q.size // 3, np.uint8)
        self.lib.oracle_grid_lookup_ndc(np.ascontiguousarray(dag, np.uint32),
                                        np.ascontiguousarray(cell_offsets, np.uint32), length, dag_levels,
                                        int(leafmasks), q, out.size, out, threads)
        return out


class Reference:
    """The reference's own CPU build and lookup (its sources compiled in place)."""

    def __init__(self, path: str = REF_SO):
        L = C.CDLL(path)
        L.ref_num_levels.argtypes = [_f32p, C.c_uint32]
        L.ref_num_levels.restype = C.c_int
        L.ref_pyramid.argtypes = [_f32p, C.c_uint32, _f32p]
        L.ref_pyramid.restype = C.c_int
        L.ref_create_childmask.argtypes = [_f32p, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_uint32]
        L.ref_create_childmask.restype = C.c_uint32
        L.ref_create.argtypes = [_f32p, C.c_uint32, C.c_uint32, C.c_uint32]
        L.ref_create.restype = C.c_void_p
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_dag_size.argtypes = [C.c_void_p]
        L.ref_dag_size.restype = C.c_size_t
        L.ref_dag_copy.argtypes = [C.c_void_p, _u32p]
        L.ref_dag_num_levels.argtypes = [C.c_void_p]
        L.ref_dag_num_levels.restype = C.c_uint32
        L.ref_total_visibility.argtypes = [C.c_void_p]
        L.ref_total_visibility.restype = C.c_int
        L.ref_traverse_ndc.argtypes = [C.c_void_p, _f32p, C.c_uint64, C.c_int, _u8p]
        L.ref_merge_level.argtypes = [_u32p, C.c_uint32, C.c_uint32, _u32p, _u32p]
        L.ref_merge_level.restype = C.c_uint32
        L.ref_grid_levels.argtypes = [C.c_uint32]
        L.ref_grid_levels.restype = C.c_uint32
        self.lib = L

    def num_levels(self, depth) -> int:
        d = np.ascontiguousarray(depth, np.float32)
        return int(self.lib.ref_num_levels(d.reshape(-1), d.shape[0]))

    def pyramid(self, depth) -> np.ndarray:
        d = np.ascontiguousarray(depth, np.float32)
        out = np.zeros(pyramid_floats(d.shape[0]), np.float32)
        self.lib.ref_pyramid(d.reshape(-1), d.shape[0], out)
        return out

    def child_mask(self, depth, level, x, y, z, z_num=1) -> int:
        d = np.ascontiguousarray(depth, np.float32)
        return int(self.lib.ref_create_childmask(d.reshape(-1), d.shape[0], level, x, y, z, z_num))

    def create(self, depth, z_index: int = 0, z_num: int = 1, ndc: np.ndarray | None = None,
               try_leafmasks: bool = True):
        """Returns (dag, num_levels, total_visibility, traverse results or None)."""
        d = np.ascontiguousarray(depth, np.float32)
        h = self.lib.ref_create(d.reshape(-1), d.shape[0], z_index, z_num)
        try:
            dag = np.zeros(self.lib.ref_dag_size(h), np.uint32)
            self.lib.ref_dag_copy(h, dag)
            nl = int(self.lib.ref_dag_num_levels(h))
            tv = int(self.lib.ref_total_visibility(h))
            vis = None
            if ndc is not None:
                q = np.ascontiguousarray(ndc, np.float32).reshape(-1)
                vis = np.zeros(q.size // 3, np.uint8)
                self.lib.ref_traverse_ndc(h, q, vis.size, int(try_leafmasks), vis)
        finally:
            self.lib.ref_free(h)
        return dag, nl, tv, vis

    def merge_level(self, words, node_size):
        w = np.ascontiguousarray(words, np.uint32)
        out = np.zeros_like(w)
        mapping = np.zeros(w.size // node_size, np.uint32)
        left = self.lib.ref_merge_level(w, w.size, node_size, out, mapping)
        return out, mapping, int(left)

    def grid_levels(self, num_cells: int) -> int:
        return int(self.lib.ref_grid_levels(num_cells))
