"""GB300 compressed precomputed shadows: Python mirror of the reference API.

The reference (TobiasRp/cpvs) exposes the shadow path as C++ classes:
``MinMaxHierarchy(const ImageF&)``, ``CompressedShadow::create(minMax,
zTileIndex, zTileNum)``, ``CompressedShadow::traverse(ndc, tryLeafmasks)``,
``getDAG()``, ``getTotalVisibility()``, ``getNumLevels()`` and
``CompressedShadowContainer``.  This package keeps those names and argument
meanings over the library's C ABI (include/cpvs.h, libcpvs_gb300.so); every
computation runs on the GPU.  The library is loaded from this directory and
is required: importing the API without it raises, there is no fallback.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcpvs_gb300.so")

SHADOW, VISIBLE, PARTIAL = 0, 1, 2
FLAG_LEAFMASKS = 0x1
IO_DEVICE = 0x100
FLAG_BORROW_INPUT = 0x200
EVAL_U8 = 0x400

STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "timed out",
          4: "CUDA device error", 5: "unimplemented", 6: "memory budget exceeded", 7: "cancelled",
          8: "output buffer too small"}


class CpvsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


# name -> (restype, argtypes)
_vp, _u32, _u64, _i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
_SIGS = {
    "cpvs_abi_version": (C.c_int, []),
    "cpvs_status_string": (C.c_char_p, [C.c_int]),
    "cpvs_last_error": (C.c_char_p, []),
    "cpvs_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "cpvs_ctx_destroy": (None, [_vp]),
    "cpvs_ctx_set_budget": (C.c_int, [_vp, _u64]),
    "cpvs_ctx_bytes_in_use": (_u64, [_vp]),
    "cpvs_ctx_set_option": (C.c_int, [_vp, C.c_int, C.c_int64]),
    "cpvs_ctx_get_option": (C.c_int64, [_vp, C.c_int]),
    "cpvs_ctx_last_build": (C.c_int, [_vp, _vp]),
    "cpvs_hierarchy_create_batch": (C.c_int, [_vp, _vp, _vp, _u32, _u32, _vp, _vp]),
    "cpvs_ctx_enable_timing": (C.c_int, [_vp, C.c_int]),
    "cpvs_ctx_kernel_times": (C.c_int, [_vp, _vp, _vp, _u32, C.POINTER(_u32)]),
    "cpvs_kernel_name": (C.c_char_p, [_u32]),
    "cpvs_raster_depth": (C.c_int, [_vp, _vp, _u32, _vp, _u32, C.c_float, _u32, _u32, _u32, _u32, _u32, _vp, _u32,
                                    _vp]),
    "cpvs_raster_triangles": (C.c_int, [_vp, _vp, _u32, C.c_float, _u32, _u32, _u32, _u32, _u32, _vp, _u32, _vp]),
    "cpvs_hierarchy_create": (C.c_int, [_vp, _vp, _u32, _u32, _vp, C.POINTER(_vp)]),
    "cpvs_hierarchy_destroy": (None, [_vp]),
    "cpvs_hierarchy_num_levels": (_u32, [_vp]),
    "cpvs_hierarchy_size": (_u32, [_vp]),
    "cpvs_hierarchy_level": (C.c_int, [_vp, _u32, _vp, _u64, _vp]),
    "cpvs_shadow_create": (C.c_int, [_vp, _vp, _u32, _u32, _u32, _vp, C.POINTER(_vp)]),
    "cpvs_shadow_create_from_depth": (C.c_int, [_vp, _vp, _u32, _u32, _u32, _u32, _vp, C.POINTER(_vp)]),
    "cpvs_shadow_destroy": (None, [_vp]),
    "cpvs_shadow_create_batch": (C.c_int, [_vp, _vp, _u32, _vp, _u32, _u32, _vp, _vp]),
    "cpvs_grid_build": (C.c_int, [_vp, _vp, _u32, _vp]),
    "cpvs_shadow_num_levels": (_u32, [_vp]),
    "cpvs_shadow_uses_leafmasks": (C.c_int, [_vp]),
    "cpvs_shadow_total_visibility": (C.c_int, [_vp]),
    "cpvs_shadow_dag_size": (_u64, [_vp]),
    "cpvs_shadow_dag_words": (C.c_int, [_vp, _vp, _u64, C.POINTER(_u64), _vp]),
    "cpvs_shadow_device_dag": (_vp, [_vp]),
    "cpvs_shadow_level_counts": (C.c_int, [_vp, _vp, _vp, _u32]),
    "cpvs_shadow_lookup_ndc": (C.c_int, [_vp, _vp, _u64, _vp, _u32, _vp]),
    "cpvs_shadow_lookup_voxel": (C.c_int, [_vp, _vp, _u64, _vp, _u32, _vp]),
    "cpvs_lookup_ndc_multi": (C.c_int, [_vp, _u32, _vp, _vp, _u64, _vp, _u32, _vp]),
    "cpvs_server_create": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "cpvs_server_destroy": (None, [_vp]),
    "cpvs_server_submit_build": (C.c_int, [_vp, _u64, _vp, _u32, C.POINTER(_u64)]),
    "cpvs_server_submit_lookup": (C.c_int, [_vp, _u64, _vp, _u64, _vp, C.POINTER(_u64)]),
    "cpvs_server_wait": (C.c_int, [_vp, _u64, C.c_int64, C.POINTER(C.c_double)]),
    "cpvs_server_cancel": (C.c_int, [_vp, _u64]),
    "cpvs_server_get_stats": (C.c_int, [_vp, _vp]),
    "cpvs_grid_create": (C.c_int, [_vp, _u32, C.POINTER(_vp)]),
    "cpvs_grid_destroy": (None, [_vp]),
    "cpvs_grid_length": (_u32, [_vp]),
    "cpvs_grid_set": (C.c_int, [_vp, _u32, _u32, _u32, _vp]),
    "cpvs_grid_get": (_vp, [_vp, _u32, _u32, _u32]),
    "cpvs_grid_finalize": (C.c_int, [_vp, C.c_int, _vp]),
    "cpvs_grid_dag_size": (_u64, [_vp]),
    "cpvs_grid_words": (C.c_int, [_vp, _vp, _u64, _vp, _u64, _vp]),
    "cpvs_grid_lookup_ndc": (C.c_int, [_vp, _vp, _u64, _vp, _u32, _vp]),
    "cpvs_grid_set_filter_size": (C.c_int, [_vp, _u32]),
    "cpvs_shadow_serialize": (C.c_int, [_vp, _vp, _u64, _vp, _vp]),
    "cpvs_shadow_deserialize": (C.c_int, [_vp, _vp, _u64, _vp, _vp]),
    "cpvs_grid_serialize": (C.c_int, [_vp, _vp, _u64, _vp, _vp]),
    "cpvs_grid_deserialize": (C.c_int, [_vp, _vp, _u64, _vp, _vp]),
    "cpvs_grid_evaluate": (C.c_int, [_vp, _vp, _u32, _u32, _u32, _vp, _u32, _vp, _vp]),
    "cpvs_shadow_build_noalloc": (C.c_int, [_vp, _u32, _u32, _u32, _u32, _vp, _u64, C.POINTER(_u64), _vp]),
    "cpvs_shade": (C.c_int, [_vp, _u32, _u32, _vp, _u32, _vp, _vp, _vp, _u32, _vp, _u32, _vp, _vp, _vp, _vp]),
}

_lib: Optional[C.CDLL] = None
_exiting = False
_servers = weakref.WeakSet()


@atexit.register
def _at_exit():
    """Servers are stopped (their threads joined) while the library is intact;
    after that, native objects still alive at interpreter exit are left to the
    process teardown instead of being destroyed in an arbitrary order."""
    global _exiting
    for srv in list(_servers):
        srv.close()
    _exiting = True


def _live() -> bool:
    return _lib is not None and not _exiting


def library_path() -> str:
    return LIB_PATH


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads libcpvs_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m cpvs_gb300.build` "
                          "(the shadow path has no CPU fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list:
    return list(_SIGS)


def _check(status: int):
    if status != 0:
        msg = _lib.cpvs_last_error().decode(errors="replace") if _lib else ""
        raise CpvsError(status, msg)


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())  # torch tensor


def _is_device(a) -> bool:
    return not isinstance(a, np.ndarray) and getattr(a, "is_cuda", False)


def _checked(a, dtype, min_elems: int, name: str, device: Optional[int] = None):
    """`a` (numpy array or torch tensor), checked as a buffer the library
    reads or writes `min_elems` elements of `dtype` through its data pointer:
    C-contiguous, of that element size and kind (float or integer), large
    enough, and -- with `device` -- a CUDA tensor on that device.  A buffer
    failing any of these would be read or written out of bounds, so it is
    refused with ValueError before the call."""
    dt = np.dtype(dtype)
    if isinstance(a, np.ndarray):
        contiguous, size, numel, is_float = a.flags.c_contiguous, a.itemsize, a.size, a.dtype.kind == "f"
    else:
        contiguous, size, numel, is_float = a.is_contiguous(), a.element_size(), a.numel(), a.dtype.is_floating_point
    if device is not None and not (_is_device(a) and a.device.index == device):
        raise ValueError(f"{name}: expected a CUDA tensor on device {device}")
    if not contiguous:
        raise ValueError(f"{name}: must be contiguous")
    if size != dt.itemsize or is_float != (dt.kind == "f"):
        raise ValueError(f"{name}: elements must be {dt.itemsize}-byte {'floats' if dt.kind == 'f' else 'integers'}")
    if numel < min_elems:
        raise ValueError(f"{name}: {numel} elements, at least {min_elems} needed")
    return a


def _host_array(a, dtype):
    """A C-contiguous host buffer for `a` without copying when it already is
    one (numpy array or CPU tensor, pinned or not)."""
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, dtype)
    if a.is_contiguous() and str(a.dtype).endswith(np.dtype(dtype).name):
        return a  # torch CPU tensor: passed by its data pointer
    return np.ascontiguousarray(a.numpy(), dtype)


def _stream(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


class Context:
    """One device (cpvs_ctx).  A process-wide default is created lazily."""

    _default: Optional["Context"] = None

    def __init__(self, device: int = 0):
        lib = load_library()
        h = _vp()
        _check(lib.cpvs_ctx_create(device, C.byref(h)))
        self.handle = h.value
        self.device = device

    @classmethod
    def default(cls) -> "Context":
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def set_budget(self, nbytes: int):
        _check(_lib.cpvs_ctx_set_budget(self.handle, int(nbytes)))

    def bytes_in_use(self) -> int:
        return int(_lib.cpvs_ctx_bytes_in_use(self.handle))

    OPT_LOOKUP_QUERIES_PER_THREAD = 1
    OPT_BUILD_CLUSTER_CAP = 2
    OPT_BUILD_INSERT_WAVES = 3

    def set_option(self, key: int, value: int):
        _check(_lib.cpvs_ctx_set_option(self.handle, key, int(value)))

    def get_option(self, key: int) -> int:
        return int(_lib.cpvs_ctx_get_option(self.handle, key))

    def last_build(self) -> dict:
        """What the last successful build did (cpvs_ctx_last_build): its
        final internal-check word (0), plan re-growths, launch shapes, and
        whether it timed the candidate shapes (a plan's first build)."""
        class _Report(C.Structure):
            _fields_ = [("error_word", C.c_uint32), ("replans", C.c_uint32), ("cluster_cap", C.c_uint32),
                        ("insert_waves", C.c_uint32), ("tuned", C.c_uint32), ("tuning_ms", C.c_float)]
        r = _Report()
        _check(_lib.cpvs_ctx_last_build(self.handle, C.byref(r)))
        return {f: getattr(r, f) for f, _ in _Report._fields_}

    def enable_timing(self, on: bool = True):
        _check(_lib.cpvs_ctx_enable_timing(self.handle, int(on)))

    def kernel_times(self) -> dict:
        """{kernel name: (total ms, launches)} since timing was enabled."""
        cap = 64
        ms = (C.c_double * cap)()
        ln = (C.c_uint64 * cap)()
        cnt = C.c_uint32()
        _check(_lib.cpvs_ctx_kernel_times(self.handle, ms, ln, cap, C.byref(cnt)))
        return {_lib.cpvs_kernel_name(i).decode(): (float(ms[i]), int(ln[i])) for i in range(cnt.value)}

    def __del__(self):
        if getattr(self, "handle", None) and _live():
            _lib.cpvs_ctx_destroy(self.handle)
            self.handle = None


def unpack_bits(words: np.ndarray, n: int) -> np.ndarray:
    """Bit-packed lookup result -> uint8 class per point (1 lit, 0 shadow)."""
    b = np.unpackbits(np.ascontiguousarray(words, np.uint32).view(np.uint8), bitorder="little")
    return b[:n].astype(np.uint8)


def raster_depth(sc, x0: int = 0, y0: int = 0, w: Optional[int] = None, h: Optional[int] = None,
                 out=None, ctx: Optional[Context] = None, stream=None):
    """Depth map of a `cpvs_gb300.scene.Scene` (or its window) rasterised on
    the GPU, into a new (h, w) float32 CUDA tensor or `out`."""
    import torch
    ctx = ctx or Context.default()
    w = sc.n if w is None else w
    h = sc.n if h is None else h
    dev = torch.device("cuda", ctx.device)
    boxes = torch.from_numpy(np.ascontiguousarray(sc.boxes, np.float32)).to(dev)
    spheres = torch.from_numpy(np.ascontiguousarray(sc.spheres, np.float32)).to(dev)
    if out is None:
        out = torch.empty((h, w), dtype=torch.float32, device=dev)
    _checked(out, np.float32, h * w, "out", ctx.device)
    nb, ns = int(sc.boxes.shape[0]), int(sc.spheres.shape[0])
    _check(_lib.cpvs_raster_depth(ctx.handle, _ptr(boxes) if nb else None, nb, _ptr(spheres) if ns else None, ns,
                                  float(sc.plane), sc.n, x0, y0, w, h, _ptr(out), IO_DEVICE, _stream(stream)))
    if stream is None:
        torch.cuda.synchronize(dev)
    return out


def shade(normals, albedo, light_direction, visibilities=None, positions=None, shadow_map=None,
          light_view_proj=None, out=None, ctx: Optional[Context] = None, stream=None):
    """The deferred shading pass (shader/shade.frag:34-56) on G-buffer
    images: (H, W, C>=3) normals, (H, W, 4) albedo and a light direction,
    with either the (H, W) uint8 visibilities of
    CompressedShadowContainer.evaluate (renderShadow on) or the plain
    shadow-map test of (H, W, C>=3) world positions against a square depth
    map under `light_view_proj` (4x4 acting on column vectors, or 16 floats
    column-major).  Returns (H, W, 4) float32 colours: a CUDA tensor for CUDA
    tensors in, else a numpy array (the images then go through the device)."""
    import torch
    ctx = ctx or Context.default()
    host = not _is_device(normals)
    dev = torch.device("cuda", ctx.device)

    def on_dev(a, dtype):
        if a is None:
            return None
        t = a if _is_device(a) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(device=dev, dtype=dtype).contiguous()

    nrm, alb = on_dev(normals, torch.float32), on_dev(albedo, torch.float32)
    h, w, fpn = (int(v) for v in nrm.shape)
    if tuple(alb.shape) != (h, w, 4):
        raise ValueError("albedo must be (H, W, 4)")
    light = np.ascontiguousarray(np.asarray(light_direction, np.float32).reshape(3))
    vis = on_dev(visibilities, torch.uint8)
    pos = sm = None
    colmajor = None
    fpp = side = 0
    if vis is None:
        pos, sm = on_dev(positions, torch.float32), on_dev(shadow_map, torch.float32)
        if pos is None or sm is None or light_view_proj is None:
            raise ValueError("without visibilities, positions, shadow_map and light_view_proj are needed")
        fpp, side = int(pos.shape[-1]), int(sm.shape[0])
        if sm.dim() != 2 or int(sm.shape[1]) != side:
            raise ValueError("shadow_map must be square")
        M = np.asarray(light_view_proj, np.float32)
        colmajor = np.ascontiguousarray(M.T.ravel() if M.shape == (4, 4) else M.ravel(), np.float32)
    elif tuple(vis.shape) != (h, w):
        raise ValueError("visibilities must be (H, W)")
    res = out if (out is not None and not host) else torch.empty((h, w, 4), dtype=torch.float32, device=dev)
    _checked(res, np.float32, h * w * 4, "out", ctx.device)
    _check(_lib.cpvs_shade(ctx.handle, w, h, _ptr(nrm), fpn, _ptr(alb), _ptr(vis) if vis is not None else None,
                           _ptr(pos) if pos is not None else None, fpp, _ptr(sm) if sm is not None else None, side,
                           colmajor.ctypes.data if colmajor is not None else None, light.ctypes.data, _ptr(res),
                           _stream(stream)))
    if host:
        return res.cpu().numpy()
    if stream is None:
        torch.cuda.synchronize(dev)
    return res


def raster_triangles(tris, n: int, plane: float, x0: int = 0, y0: int = 0, w: Optional[int] = None,
                     h: Optional[int] = None, ctx: Optional[Context] = None, stream=None):
    """Depth map of (m, 9) float32 triangles (x0,y0,d0, x1,y1,d1, x2,y2,d2 in map
    coordinates) over a plane, rasterised on the GPU (cpvs_raster_triangles).
    numpy in -> numpy (h, w) out; CUDA tensor in -> CUDA tensor out."""
    ctx = ctx or Context.default()
    w = n if w is None else w
    h = n if h is None else h
    m = int(tris.shape[0])
    if _is_device(tris):
        import torch
        _checked(tris, np.float32, 9 * m, "tris", ctx.device)
        out = torch.empty((h, w), dtype=torch.float32, device=tris.device)
        _check(_lib.cpvs_raster_triangles(ctx.handle, _ptr(tris) if m else None, m, float(plane), n, x0, y0, w, h,
                                          _ptr(out), IO_DEVICE, _stream(stream)))
        return out
    t = _checked(np.ascontiguousarray(tris, np.float32), np.float32, 9 * m, "tris")
    out = np.empty((h, w), np.float32)
    _check(_lib.cpvs_raster_triangles(ctx.handle, t.ctypes.data if m else None, m, float(plane), n, x0, y0, w, h,
                                      out.ctypes.data, 0, _stream(stream)))
    return out


class MinMaxHierarchy:
    """Device min-max pyramid of a square power-of-two depth map
    (src/MinMaxHierarchy.h:12-92).  `depth` is an (n, n) float32 numpy array
    or CUDA tensor."""

    def __init__(self, depth, ctx: Optional[Context] = None, stream=None, borrow: bool = False):
        """`borrow` (CUDA tensor input only): read the map in place instead of
        copying it; the tensor is kept referenced for the hierarchy's life and
        must not be modified meanwhile."""
        self.ctx = ctx or Context.default()
        n = int(depth.shape[0])
        if tuple(depth.shape) != (n, n):
            raise ValueError("depth map must be square")
        dev = _is_device(depth)
        if not dev:
            depth = _host_array(depth, np.float32)
        else:
            _checked(depth, np.float32, n * n, "depth", self.ctx.device)
        flags = (IO_DEVICE | (FLAG_BORROW_INPUT if borrow else 0)) if dev else 0
        self._borrowed = depth if (dev and borrow) else None
        h = _vp()
        _check(_lib.cpvs_hierarchy_create(self.ctx.handle, _ptr(depth), n, flags, _stream(stream), C.byref(h)))
        self.handle = h.value
        self.n = n
        self._levels = {}

    @classmethod
    def create_batch(cls, maps, ctx: Optional[Context] = None, stream=None, borrow: bool = False) -> list:
        """One hierarchy per map (cpvs_hierarchy_create_batch): the maps'
        pyramids in one launch per pass.  `maps`: square power-of-two float32
        maps, all numpy arrays or all CUDA tensors (`borrow` as in the
        constructor)."""
        maps = list(maps)
        if not maps:
            return []
        dev = _is_device(maps[0])
        if any(_is_device(m) != dev for m in maps):
            raise ValueError("create_batch: maps must all be host arrays or all CUDA tensors")
        for m in maps:
            if len(m.shape) != 2 or m.shape[0] != m.shape[1]:
                raise ValueError("depth map must be square")
        ctx = ctx or Context.default()
        keep = []
        for m in maps:
            n = int(m.shape[0])
            if dev:
                if not m.is_contiguous():
                    raise ValueError("device depth map must be contiguous")
                _checked(m, np.float32, n * n, "map", ctx.device)
                keep.append(m)
            else:
                keep.append(_host_array(m, np.float32))
        ptrs = (_vp * len(keep))(*[_ptr(m) for m in keep])
        sides = (_u32 * len(keep))(*[int(m.shape[0]) for m in keep])
        out = (_vp * len(keep))()
        flags = (IO_DEVICE | (FLAG_BORROW_INPUT if borrow else 0)) if dev else 0
        _check(_lib.cpvs_hierarchy_create_batch(ctx.handle, ptrs, sides, len(keep), flags, _stream(stream), out))
        hs = []
        for i, m in enumerate(keep):
            h = cls.__new__(cls)
            h.ctx = ctx
            h._borrowed = m if (dev and borrow) else None
            h.handle = out[i]
            h.n = int(m.shape[0])
            h._levels = {}
            hs.append(h)
        return hs

    def get_num_levels(self) -> int:
        return int(_lib.cpvs_hierarchy_num_levels(self.handle))

    getNumLevels = get_num_levels

    def level(self, level: int) -> np.ndarray:
        """(s, s, 2) array of (min, max) of pyramid level `level` >= 1."""
        if level not in self._levels:
            s = self.n >> level
            out = np.zeros((s, s, 2), np.float32)
            _check(_lib.cpvs_hierarchy_level(self.handle, level, out.ctypes.data, out.size, 0))
            self._levels[level] = out
        return self._levels[level]

    def get_min(self, level: int, x: int, y: int) -> float:
        return float(self.level(level)[y, x, 0])

    def get_max(self, level: int, x: int, y: int) -> float:
        return float(self.level(level)[y, x, 1])

    getMin, getMax = get_min, get_max

    def __del__(self):
        if getattr(self, "handle", None) and _live():
            _lib.cpvs_hierarchy_destroy(self.handle)
            self.handle = None


class _BuildJob(C.Structure):
    _fields_ = [("source", C.c_uint32), ("z_tile_index", C.c_uint32), ("z_tile_num", C.c_uint32)]


class CompressedShadow:
    """A resident shadow DAG (src/CompressedShadow.h:20-125)."""

    SHADOW, VISIBLE, PARTIAL = SHADOW, VISIBLE, PARTIAL

    def __init__(self, handle: int, ctx: Context, owned: bool = True):
        self.handle = handle
        self.ctx = ctx
        self._owned = owned
        self._dag = None

    @staticmethod
    def create(min_max: MinMaxHierarchy, z_tile_index: int = 0, z_tile_num: int = 1, leafmasks: bool = True,
               stream=None) -> "CompressedShadow":
        """CompressedShadow::create(minMax, zTileIndex, zTileNum)."""
        h = _vp()
        _check(_lib.cpvs_shadow_create(min_max.ctx.handle, min_max.handle, z_tile_index, z_tile_num,
                                       FLAG_LEAFMASKS if leafmasks else 0, _stream(stream), C.byref(h)))
        return CompressedShadow(h.value, min_max.ctx)

    @staticmethod
    def from_depth(depth, z_tile_index: int = 0, z_tile_num: int = 1, leafmasks: bool = True,
                   ctx: Optional[Context] = None, stream=None) -> "CompressedShadow":
        """CompressedShadow::create(const ShadowMap*, ...): depth map -> DAG."""
        n = int(depth.shape[0])
        if tuple(depth.shape) != (n, n):
            raise ValueError("depth map must be square")
        ctx = ctx or Context.default()
        dev = _is_device(depth)
        if dev:
            _checked(depth, np.float32, n * n, "depth", ctx.device)
        else:
            depth = _host_array(depth, np.float32)
        flags = (FLAG_LEAFMASKS if leafmasks else 0) | (IO_DEVICE if dev else 0)
        h = _vp()
        _check(_lib.cpvs_shadow_create_from_depth(ctx.handle, _ptr(depth), n, z_tile_index, z_tile_num, flags,
                                                  _stream(stream), C.byref(h)))
        return CompressedShadow(h.value, ctx)

    def to_bytes(self, stream=None) -> bytes:
        """The saved form (cpvs_shadow_serialize): header, level counts, DAG."""
        size = C.c_uint64()
        _check(_lib.cpvs_shadow_serialize(self.handle, None, 0, C.byref(size), _stream(stream)))
        buf = np.zeros(size.value, np.uint8)
        _check(_lib.cpvs_shadow_serialize(self.handle, buf.ctypes.data, buf.size, C.byref(size), _stream(stream)))
        return buf.tobytes()

    @staticmethod
    def from_bytes(data, ctx: Optional[Context] = None, stream=None) -> "CompressedShadow":
        ctx = ctx or Context.default()
        buf = np.frombuffer(data, np.uint8)
        h = _vp()
        _check(_lib.cpvs_shadow_deserialize(ctx.handle, buf.ctypes.data, buf.size, _stream(stream), C.byref(h)))
        return CompressedShadow(h.value, ctx)

    def save(self, path: str):
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @staticmethod
    def load(path: str, ctx: Optional[Context] = None) -> "CompressedShadow":
        with open(path, "rb") as f:
            return CompressedShadow.from_bytes(f.read(), ctx)

    @staticmethod
    def create_batch(sources, jobs, leafmasks: bool = True, stream=None) -> list:
        """Many DAGs in one batch.  `sources`: MinMaxHierarchy list; `jobs`:
        (source index, z_tile_index, z_tile_num) per DAG.  Returns one
        CompressedShadow per job."""
        sources, jobs = list(sources), list(jobs)
        if not jobs:
            return []
        if not sources:
            raise ValueError("create_batch: no sources")
        ctx = sources[0].ctx
        hs = (_vp * len(sources))(*[m.handle for m in sources])
        jb = (_BuildJob * len(jobs))(*[_BuildJob(*j) for j in jobs])
        out = (_vp * len(jobs))()
        _check(_lib.cpvs_shadow_create_batch(ctx.handle, hs, len(sources), jb, len(jobs),
                                             FLAG_LEAFMASKS if leafmasks else 0, _stream(stream), out))
        return [CompressedShadow(out[j], ctx) for j in range(len(jobs))]

    def get_num_levels(self) -> int:
        return int(_lib.cpvs_shadow_num_levels(self.handle))

    def uses_leafmasks(self) -> bool:
        return bool(_lib.cpvs_shadow_uses_leafmasks(self.handle))

    def get_total_visibility(self) -> int:
        return int(_lib.cpvs_shadow_total_visibility(self.handle))

    def dag_size(self) -> int:
        return int(_lib.cpvs_shadow_dag_size(self.handle))

    def get_dag(self, out=None, stream=None):
        """CompressedShadow::getDAG(): the DAG words, copied to the host (and
        cached).  With `out` (a host uint32 array or tensor of at least
        dag_size() words, e.g. reused pinned memory) the words are written
        there and a view of it is returned, uncached."""
        if out is not None:
            n = self.dag_size()
            if _is_device(out):
                raise ValueError("get_dag: out must be host memory")
            _checked(out, np.uint32, n, "get_dag: out")
            _check(_lib.cpvs_shadow_dag_words(self.handle, _ptr(out), n, None, _stream(stream)))
            return out[:n]
        if self._dag is None:
            n = self.dag_size()
            buf = np.zeros(max(n, 1), np.uint32)
            _check(_lib.cpvs_shadow_dag_words(self.handle, buf.ctypes.data, buf.size, None, _stream(stream)))
            self._dag = buf[:n]
        return self._dag

    getNumLevels, getTotalVisibility, getDAG = get_num_levels, get_total_visibility, get_dag

    def device_dag(self) -> int:
        return int(_lib.cpvs_shadow_device_dag(self.handle) or 0)

    def level_counts(self):
        nl = self.get_num_levels()
        t = np.zeros(nl, np.uint64)
        u = np.zeros(nl, np.uint64)
        _check(_lib.cpvs_shadow_level_counts(self.handle, t.ctypes.data, u.ctypes.data, nl))
        return t.astype(np.int64).tolist(), u.astype(np.int64).tolist()

    def lookup_ndc(self, points, out=None, stream=None):
        """Visibility of (n, 3) float32 NDC points.  numpy in -> uint8 classes
        out; CUDA tensor in -> bit-packed int32 CUDA tensor out."""
        return self._lookup(points, True, out, stream)

    def lookup_voxel(self, points, out=None, stream=None):
        """Visibility of (n, 3) int32 voxel coordinates."""
        return self._lookup(points, False, out, stream)

    def _lookup(self, points, ndc: bool, out, stream):
        fn = _lib.cpvs_shadow_lookup_ndc if ndc else _lib.cpvs_shadow_lookup_voxel
        n = int(points.shape[0])
        if _is_device(points):
            import torch
            if out is None:
                out = torch.empty((n + 31) // 32, dtype=torch.int32, device=points.device)
            _checked(points, np.float32 if ndc else np.int32, 3 * n, "points", self.ctx.device)
            _checked(out, np.int32, (n + 31) // 32, "out", self.ctx.device)
            _check(fn(self.handle, _ptr(points), n, _ptr(out), IO_DEVICE, _stream(stream)))
            return out
        pts = _checked(np.ascontiguousarray(points, np.float32 if ndc else np.int32), np.float32 if ndc else np.int32,
                       3 * n, "points")
        words = np.zeros(max((n + 31) // 32, 1), np.uint32)
        _check(fn(self.handle, pts.ctypes.data, n, words.ctypes.data, 0, _stream(stream)))
        return unpack_bits(words, n)

    def lookup_ndc_packed(self, points, words_out, stream=None):
        """Host-buffer lookup: (n, 3) float32 host points (numpy or CPU
        tensor, pinned for asynchronous copies) -> bit-packed words written to
        the host buffer `words_out` (ceil(n/32) 32-bit words).  The copies in
        and out happen inside the call."""
        n = int(points.shape[0])
        pts = _host_array(points, np.float32)
        if _is_device(words_out):
            raise ValueError("words_out must be host memory")
        _checked(pts, np.float32, 3 * n, "points")
        _checked(words_out, np.uint32, (n + 31) // 32, "words_out")
        _check(_lib.cpvs_shadow_lookup_ndc(self.handle, _ptr(pts), n, _ptr(words_out), 0, _stream(stream)))
        return words_out

    def traverse(self, position, try_leafmasks: bool = True) -> int:
        """CompressedShadow::traverse(ndc, tryLeafmasks) for one point (a
        one-element GPU lookup; batch with lookup_ndc).  `try_leafmasks` must
        match how the DAG was built, as in the reference."""
        if bool(try_leafmasks) != self.uses_leafmasks():
            raise ValueError("try_leafmasks must match the DAG's leafmask mode")
        return int(self.lookup_ndc(np.asarray(position, np.float32).reshape(1, 3))[0])

    def release(self):
        if getattr(self, "handle", None) and self._owned and _live():
            _lib.cpvs_shadow_destroy(self.handle)
        self.handle = None

    def __del__(self):
        self.release()


def lookup_ndc_multi(shadows, dag_index, points, out=None, stream=None):
    """Point i looked up in shadows[dag_index[i]] in one launch.  numpy in ->
    uint8 classes out; CUDA tensors in -> bit-packed int32 CUDA tensor out."""
    n = int(points.shape[0])
    tab = (_vp * len(shadows))(*[s.handle for s in shadows])
    if _is_device(points):
        import torch
        if out is None:
            out = torch.empty((n + 31) // 32, dtype=torch.int32, device=points.device)
        dev = points.device.index
        _checked(points, np.float32, 3 * n, "points", dev)
        _checked(dag_index, np.uint32, n, "dag_index", dev)
        _checked(out, np.int32, (n + 31) // 32, "out", dev)
        _check(_lib.cpvs_lookup_ndc_multi(tab, len(shadows), _ptr(dag_index), _ptr(points), n, _ptr(out), IO_DEVICE,
                                          _stream(stream)))
        return out
    pts = _host_array(points, np.float32)
    ids = _host_array(dag_index, np.uint32)
    _checked(pts, np.float32, 3 * n, "points")
    _checked(ids, np.uint32, n, "dag_index")
    words = np.zeros(max((n + 31) // 32, 1), np.uint32)
    _check(_lib.cpvs_lookup_ndc_multi(tab, len(shadows), _ptr(ids), _ptr(pts), n, words.ctypes.data, 0,
                                      _stream(stream)))
    return unpack_bits(words, n)


class CompressedShadowContainer:
    """Cubic length^3 top-level grid of DAGs (src/CompressedShadowContainer.h:21-73)."""

    def __init__(self, length: int = 1, ctx: Optional[Context] = None):
        self.ctx = ctx or Context.default()
        h = _vp()
        _check(_lib.cpvs_grid_create(self.ctx.handle, length, C.byref(h)))
        self.handle = h.value
        self.length = length
        self._cells = {}

    @classmethod
    def of(cls, shadow: CompressedShadow) -> "CompressedShadowContainer":
        c = cls(1, shadow.ctx)
        c.set(shadow, 0, 0, 0)
        return c

    def set(self, shadow: CompressedShadow, x: int, y: int, z: int):
        """Cell (x,y,z) takes ownership of the shadow (the reference moves a
        unique_ptr in): the shadow object stays usable while the container
        holds it, and is released with the container, when its cell is
        replaced, or by move_to_gpu and build.  A released shadow, or one that
        a cell already holds, is refused."""
        if getattr(shadow, "handle", None) is None:
            raise ValueError("set: the shadow has been released (its container took it)")
        if not shadow._owned and self._cells.get((x, y, z)) is not shadow:
            raise ValueError("set: the shadow already belongs to a container cell")
        _check(_lib.cpvs_grid_set(self.handle, x, y, z, shadow.handle))
        old = self._cells.get((x, y, z))
        if old is not None and old is not shadow:
            old.handle = None  # destroyed by the grid
        shadow._owned = False
        self._cells[(x, y, z)] = shadow

    def _release_cells(self):
        for s in self._cells.values():
            s.handle = None
        self._cells.clear()

    def get(self, x: int, y: int, z: int) -> Optional[CompressedShadow]:
        return self._cells.get((x, y, z))

    def build(self, xy_tiles, leafmasks: bool = True, stream=None):
        """Builds every cell in one batch: cell (x,y,z) = z-tile z of
        xy_tiles[y*length+x] (MinMaxHierarchy objects of one size)."""
        xy_tiles = list(xy_tiles)
        if len(xy_tiles) != self.length ** 2:
            raise ValueError(f"build: needs length^2 = {self.length ** 2} xy tiles, got {len(xy_tiles)}")
        hs = (_vp * len(xy_tiles))(*[m.handle for m in xy_tiles])
        _check(_lib.cpvs_grid_build(self.handle, hs, FLAG_LEAFMASKS if leafmasks else 0, _stream(stream)))
        self._release_cells()  # the grid destroyed the cells' previous shadows

    def copy_to_gpu(self, stream=None):
        _check(_lib.cpvs_grid_finalize(self.handle, 0, _stream(stream)))

    def move_to_gpu(self, stream=None):
        _check(_lib.cpvs_grid_finalize(self.handle, 1, _stream(stream)))
        self._release_cells()

    copyToGPU, moveToGPU = copy_to_gpu, move_to_gpu

    def words(self):
        """(combined DAG words, per-cell words) after copy_to_gpu."""
        n = int(_lib.cpvs_grid_dag_size(self.handle))
        dag = np.zeros(max(n, 1), np.uint32)
        cells = np.zeros(self.length ** 3, np.uint32)
        _check(_lib.cpvs_grid_words(self.handle, dag.ctypes.data, dag.size, cells.ctypes.data, cells.size, 0))
        return dag[:n], cells

    def lookup_ndc(self, points, out=None, stream=None):
        n = int(points.shape[0])
        if _is_device(points):
            import torch
            if out is None:
                out = torch.empty((n + 31) // 32, dtype=torch.int32, device=points.device)
            _checked(points, np.float32, 3 * n, "points", self.ctx.device)
            _checked(out, np.int32, (n + 31) // 32, "out", self.ctx.device)
            _check(_lib.cpvs_grid_lookup_ndc(self.handle, _ptr(points), n, _ptr(out), IO_DEVICE, _stream(stream)))
            return out
        pts = _checked(np.ascontiguousarray(points, np.float32), np.float32, 3 * n, "points")
        words = np.zeros(max((n + 31) // 32, 1), np.uint32)
        _check(_lib.cpvs_grid_lookup_ndc(self.handle, pts.ctypes.data, n, words.ctypes.data, 0, _stream(stream)))
        return unpack_bits(words, n)

    def to_bytes(self, stream=None) -> bytes:
        """The saved form (cpvs_grid_serialize): header, cell words, combined DAG."""
        size = C.c_uint64()
        _check(_lib.cpvs_grid_serialize(self.handle, None, 0, C.byref(size), _stream(stream)))
        buf = np.zeros(size.value, np.uint8)
        _check(_lib.cpvs_grid_serialize(self.handle, buf.ctypes.data, buf.size, C.byref(size), _stream(stream)))
        return buf.tobytes()

    @classmethod
    def from_bytes(cls, data, ctx: Optional[Context] = None, stream=None) -> "CompressedShadowContainer":
        """A finalized container (no cell shadows) from its saved form."""
        ctx = ctx or Context.default()
        buf = np.frombuffer(data, np.uint8)
        h = _vp()
        _check(_lib.cpvs_grid_deserialize(ctx.handle, buf.ctypes.data, buf.size, _stream(stream), C.byref(h)))
        c = cls.__new__(cls)
        c.ctx, c.handle, c._cells = ctx, h.value, {}
        c.length = int(_lib.cpvs_grid_length(c.handle))
        return c

    def save(self, path: str):
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @classmethod
    def load(cls, path: str, ctx: Optional[Context] = None) -> "CompressedShadowContainer":
        with open(path, "rb") as f:
            return cls.from_bytes(f.read(), ctx)

    def set_filter_size(self, size: int):
        """Width (= height) of the percentage-closer filter of evaluate."""
        _check(_lib.cpvs_grid_set_filter_size(self.handle, size))
        self.filter_size = size

    setFilterSize = set_filter_size

    def evaluate(self, positions, light_view_proj, out=None, packed: bool = False, stream=None):
        """Visibility of every world-space position of an (H, W, C>=3)
        float32 image under `light_view_proj` (4x4, M[row, col] acting on
        column vectors; a flat 16-vector is read column-major, as
        glm::value_ptr gives it).  Returns an (H, W) uint8 image (255 lit,
        0 shadowed, or the PCF fraction * 255), or with `packed` the bit
        words (filter size 1 only).  Device tensors in, device tensor out."""
        M = np.asarray(light_view_proj, np.float32)
        colmajor = np.ascontiguousarray(M.T.ravel() if M.shape == (4, 4) else M.ravel(), np.float32)
        if colmajor.size != 16:
            raise ValueError("light_view_proj must be 4x4 or 16 floats")
        h, w, fpp = (int(v) for v in positions.shape)
        n = h * w
        flags = 0 if packed else EVAL_U8
        if _is_device(positions):
            import torch
            if out is None:
                out = (torch.empty((n + 31) // 32, dtype=torch.int32, device=positions.device) if packed
                       else torch.empty((h, w), dtype=torch.uint8, device=positions.device))
            _checked(positions, np.float32, n * fpp, "positions", self.ctx.device)
            if packed:
                _checked(out, np.int32, (n + 31) // 32, "out", self.ctx.device)
            else:
                _checked(out, np.uint8, n, "out", self.ctx.device)
            _check(_lib.cpvs_grid_evaluate(self.handle, _ptr(positions), w, h, fpp, colmajor.ctypes.data,
                                           flags | IO_DEVICE, _ptr(out), _stream(stream)))
            return out
        pos = np.ascontiguousarray(positions, np.float32)
        res = np.zeros(max((n + 31) // 32, 1), np.uint32) if packed else np.zeros((h, w), np.uint8)
        _check(_lib.cpvs_grid_evaluate(self.handle, pos.ctypes.data, w, h, fpp, colmajor.ctypes.data, flags,
                                       res.ctypes.data, _stream(stream)))
        return res

    def __del__(self):
        if getattr(self, "handle", None) and _live():
            self._release_cells()
            _lib.cpvs_grid_destroy(self.handle)
            self.handle = None


class _ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_batch_builds", C.c_uint32), ("max_batch_lookups", C.c_uint32),
                ("flags", C.c_uint32)]


class _ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("builds_done", "lookups_done", "failed", "cancelled", "evictions",
                                           "resident_dags", "resident_bytes", "queued")] + \
               [(k, C.c_double) for k in ("build_p50_ms", "build_p99_ms", "lookup_p50_ms", "lookup_p99_ms")]


class Server:
    """The serving loop (cpvs_server): submit builds and lookups from any
    thread, wait on tickets.  The server takes over its context."""

    def __init__(self, ctx: Optional[Context] = None, budget_bytes: int = 0, max_batch_builds: int = 0,
                 max_batch_lookups: int = 0, leafmasks: bool = True):
        self.ctx = ctx or Context(0)
        cfg = _ServerConfig(budget_bytes, max_batch_builds, max_batch_lookups, FLAG_LEAFMASKS if leafmasks else 0)
        h = _vp()
        _check(_lib.cpvs_server_create(self.ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value
        _servers.add(self)
        self._keep = {}  # ticket -> buffers that must outlive it

    def submit_build(self, key: int, depth) -> int:
        """Queues a build of the square host map `depth` into DAG `key`."""
        if _is_device(depth):
            raise ValueError("submit_build: the depth map must be in host memory")
        if len(depth.shape) != 2 or depth.shape[0] != depth.shape[1]:
            raise ValueError("depth map must be square")
        n = int(depth.shape[0])
        d = _checked(_host_array(depth, np.float32), np.float32, n * n, "depth")
        t = C.c_uint64()
        _check(_lib.cpvs_server_submit_build(self.handle, key, _ptr(d), n, C.byref(t)))
        self._keep[t.value] = (d,)
        return t.value

    def submit_lookup(self, key: int, points, out=None) -> int:
        """Queues a lookup of the (n, 3) host points in DAG `key`; `out`, if
        given, is a host uint32 buffer of at least ceil(n/32) words."""
        if _is_device(points) or (out is not None and _is_device(out)):
            raise ValueError("submit_lookup: points and out must be in host memory")
        n = int(points.shape[0])
        pts = _checked(_host_array(points, np.float32), np.float32, 3 * n, "points")
        words = out if out is not None else np.zeros(max((n + 31) // 32, 1), np.uint32)
        _checked(words, np.uint32, (n + 31) // 32, "out")
        t = C.c_uint64()
        _check(_lib.cpvs_server_submit_lookup(self.handle, key, _ptr(pts), n, _ptr(words), C.byref(t)))
        self._keep[t.value] = (pts, words, n)
        return t.value

    def wait(self, ticket: int, timeout_us: int = -1, packed: bool = False):
        """Returns (latency_ms, result): result is the uint8 classes for a
        lookup ticket (with `packed`, the uint32 bit words as written), None
        for a build.  Raises CpvsError on failure."""
        lat = C.c_double()
        st = _lib.cpvs_server_wait(self.handle, ticket, timeout_us, C.byref(lat))
        keep = self._keep.pop(ticket, None) if st != 3 else self._keep.get(ticket)
        _check(st)
        if keep is not None and len(keep) == 3:
            if packed:
                return lat.value, keep[1]
            return lat.value, unpack_bits(np.asarray(keep[1]).view(np.uint32), keep[2])
        return lat.value, None

    def cancel(self, ticket: int):
        _check(_lib.cpvs_server_cancel(self.handle, ticket))

    def stats(self) -> dict:
        st = _ServerStats()
        _check(_lib.cpvs_server_get_stats(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "handle", None) and _live():
            _lib.cpvs_server_destroy(self.handle)
        self.handle = None

    def __del__(self):
        self.close()
