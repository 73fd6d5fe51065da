"""The C ABI library without a GPU: it builds, loads, exports exactly what
include/cpvs.h declares, and rejects bad arguments before touching the
device.  No compute call runs here."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cpvs.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^CPVS_API\s+[^(]*?\b(cpvs_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from cpvs_gb300 import build
    build.build()
    import cpvs_gb300
    return cpvs_gb300.load_library()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert len(names) >= 30
    for must in ("cpvs_shadow_create", "cpvs_shadow_lookup_ndc", "cpvs_grid_lookup_ndc", "cpvs_hierarchy_create"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    from cpvs_gb300 import LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (cpvs_\w+)$", out, re.M))
    declared = set(declared_symbols())
    assert declared <= exported, sorted(declared - exported)
    # nothing else escapes the library's C ABI
    assert exported <= declared, sorted(exported - declared)
    for name in declared:
        assert getattr(lib, name) is not None


def test_python_mirror_binds_every_symbol():
    import cpvs_gb300
    assert sorted(cpvs_gb300.exported_symbols()) == declared_symbols()


def test_status_strings_and_version(lib):
    assert lib.cpvs_abi_version() == 1
    assert lib.cpvs_status_string(0) == b"ok"
    assert lib.cpvs_status_string(6) == b"memory budget exceeded"


def test_null_arguments_are_rejected(lib):
    import ctypes as C
    h = C.c_void_p()
    assert lib.cpvs_hierarchy_create(None, None, 64, 0, None, C.byref(h)) == 1
    assert lib.cpvs_hierarchy_create_batch(None, None, None, 2, 0, None, C.byref(h)) == 1
    assert lib.cpvs_shadow_create(None, None, 0, 1, 1, None, C.byref(h)) == 1
    assert lib.cpvs_grid_create(None, 4, C.byref(h)) == 1
    assert b"null" in lib.cpvs_last_error()
    assert lib.cpvs_shadow_lookup_ndc(None, None, 0, None, 0, None) == 1
    assert lib.cpvs_shadow_num_levels(None) == 0


def test_no_device_is_an_error_not_a_fallback(lib):
    import ctypes as C
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.cpvs_ctx_create(0, C.byref(h)) == 4   # CPVS_ERR_DEVICE
    assert not h.value


def test_python_buffers_are_checked_before_the_call():
    """Buffers the library would read or write by pointer are refused when
    they are too small, strided, of the wrong element type, or not where the
    call needs them -- before any device work."""
    import numpy as np
    import torch
    from cpvs_gb300 import _checked
    a = np.zeros((4, 3), np.float32)
    assert _checked(a, np.float32, 12, "a") is a
    with pytest.raises(ValueError, match="at least"):
        _checked(a, np.float32, 13, "a")
    with pytest.raises(ValueError, match="contiguous"):
        _checked(np.zeros((3, 4), np.float32).T, np.float32, 12, "a")
    with pytest.raises(ValueError, match="floats"):
        _checked(np.zeros(12, np.int32), np.float32, 12, "a")
    with pytest.raises(ValueError, match="integers"):
        _checked(np.zeros(12, np.float32), np.uint32, 12, "a")
    with pytest.raises(ValueError, match="1-byte"):
        _checked(np.zeros(12, np.int32), np.uint8, 12, "a")
    t = torch.zeros(8, dtype=torch.int32)
    assert _checked(t, np.uint32, 8, "t") is t
    with pytest.raises(ValueError, match="CUDA tensor"):
        _checked(t, np.uint32, 8, "t", device=0)
    with pytest.raises(ValueError, match="contiguous"):
        _checked(torch.zeros(4, 4)[:, 1], np.float32, 4, "t")


def test_hierarchy_batch_checks_maps_before_any_device_work():
    """MinMaxHierarchy.create_batch refuses non-square maps before it touches
    a context; an empty batch is empty."""
    import numpy as np
    import cpvs_gb300 as cp
    assert cp.MinMaxHierarchy.create_batch([]) == []
    with pytest.raises(ValueError, match="square"):
        cp.MinMaxHierarchy.create_batch([np.zeros((8, 8), np.float32), np.zeros((4, 8), np.float32)])
    with pytest.raises(ValueError, match="square"):
        cp.MinMaxHierarchy.create_batch([np.zeros(16, np.float32)])


def test_batch_builds_check_their_lists_before_any_device_work():
    """cpvs_grid_build reads length^2 tile handles with no count beside them,
    so the Python mirror checks the count itself; a shadow batch with no jobs
    is empty and one with no sources is refused."""
    import types
    import cpvs_gb300 as cp
    with pytest.raises(ValueError, match=r"length\^2 = 4 xy tiles, got 3"):
        cp.CompressedShadowContainer.build(types.SimpleNamespace(length=2), [object()] * 3)
    assert cp.CompressedShadow.create_batch([], []) == []
    with pytest.raises(ValueError, match="no sources"):
        cp.CompressedShadow.create_batch([], [(0, 0, 1)])


def test_host_inputs_are_checked_by_shape(lib):
    """Maps, points and triangles whose shape holds fewer values than the
    call reads are refused before the call."""
    import types
    import numpy as np
    import cpvs_gb300 as cp
    with pytest.raises(ValueError, match="square"):
        cp.CompressedShadow.from_depth(np.zeros((4, 8), np.float32))
    fake = types.SimpleNamespace(handle=None, ctx=types.SimpleNamespace(handle=None, device=0))
    with pytest.raises(ValueError, match="points: 128 elements, at least 192"):
        cp.CompressedShadow._lookup(fake, np.zeros((64, 2), np.float32), True, None, None)
    with pytest.raises(ValueError, match="points: 128 elements, at least 192"):
        cp.CompressedShadow._lookup(fake, np.zeros((64, 2), np.int32), False, None, None)
    with pytest.raises(ValueError, match="points: 128 elements, at least 192"):
        cp.CompressedShadowContainer.lookup_ndc(fake, np.zeros((64, 2), np.float32))
    with pytest.raises(ValueError, match="tris: 24 elements, at least 36"):
        cp.raster_triangles(np.zeros((4, 6), np.float32), 64, 0.5, ctx=fake.ctx)
    # well-formed inputs pass the checks and meet the null handles in the library
    for call in (lambda: cp.CompressedShadow._lookup(fake, np.zeros((64, 3), np.float32), True, None, None),
                 lambda: cp.CompressedShadow._lookup(fake, np.zeros((64, 3), np.int32), False, None, None),
                 lambda: cp.CompressedShadowContainer.lookup_ndc(fake, np.zeros((64, 3), np.float32)),
                 lambda: cp.raster_triangles(np.zeros((4, 9), np.float32), 64, 0.5, ctx=fake.ctx)):
        with pytest.raises(cp.CpvsError) as e:
            call()
        assert e.value.status == 1


class _DeviceLike:
    """Stands in for a CUDA tensor on device 0 (host memory behind it), so the
    mirror's device-input checks run without a GPU.  A call that gets past
    them reaches the C ABI with a null context and is refused there."""
    is_cuda = True

    def __init__(self, arr):
        import types
        self.a = arr
        self.shape = arr.shape
        self.device = types.SimpleNamespace(index=0)
        self.dtype = types.SimpleNamespace(is_floating_point=arr.dtype.kind == "f")

    def is_contiguous(self):
        return self.a.flags.c_contiguous

    def element_size(self):
        return self.a.itemsize

    def numel(self):
        return self.a.size

    def data_ptr(self):
        return self.a.ctypes.data


def test_device_maps_are_checked_before_the_call(lib):
    """A square float32 contiguous device map passes the checks (and meets
    the null context in the library); a map of another element type, a
    strided one or one on another device is refused first."""
    import types
    import numpy as np
    import cpvs_gb300 as cp
    ctx = types.SimpleNamespace(handle=None, device=0)
    good = _DeviceLike(np.zeros((64, 64), np.float32))
    for make in (lambda d: cp.CompressedShadow.from_depth(d, ctx=ctx), lambda d: cp.MinMaxHierarchy(d, ctx=ctx)):
        with pytest.raises(cp.CpvsError, match="null argument") as e:
            make(good)
        assert e.value.status == 1
        with pytest.raises(ValueError, match="4-byte floats"):
            make(_DeviceLike(np.zeros((64, 64), np.float64)))
        with pytest.raises(ValueError, match="contiguous"):
            make(_DeviceLike(np.zeros((64, 128), np.float32)[:, ::2]))
    other = types.SimpleNamespace(handle=None, device=1)
    with pytest.raises(ValueError, match="device 1"):
        cp.CompressedShadow.from_depth(good, ctx=other)
    with pytest.raises(ValueError, match="device 1"):
        cp.MinMaxHierarchy(good, ctx=other)


def test_server_checks_its_buffers_before_any_device_work(lib):
    """The server reads the map and points and writes the bits after submit
    returns, from its own thread, so a buffer too small for the request is
    refused at submission."""
    import types
    import numpy as np
    import cpvs_gb300 as cp
    srv = types.SimpleNamespace(handle=None, _keep={})
    with pytest.raises(ValueError, match="square"):
        cp.Server.submit_build(srv, 0, np.zeros((4, 8), np.float32))
    with pytest.raises(ValueError, match="points"):
        cp.Server.submit_lookup(srv, 0, np.zeros((64, 2), np.float32))
    with pytest.raises(ValueError, match="out: 1 elements, at least 2"):
        cp.Server.submit_lookup(srv, 0, np.zeros((64, 3), np.float32), np.zeros(1, np.uint32))
    with pytest.raises(ValueError, match="integers"):
        cp.Server.submit_lookup(srv, 0, np.zeros((64, 3), np.float32), np.zeros(2, np.float32))
    # well-formed requests pass the checks and meet the null server in the library
    for call in (lambda: cp.Server.submit_build(srv, 0, np.zeros((64, 64), np.float32)),
                 lambda: cp.Server.submit_lookup(srv, 0, np.zeros((64, 3), np.float32)),
                 lambda: cp.Server.submit_lookup(srv, 0, np.zeros((64, 3), np.float32), np.zeros(2, np.uint32))):
        with pytest.raises(cp.CpvsError) as e:
            call()
        assert e.value.status == 1


@pytest.mark.gpu
def test_hierarchy_batch_refuses_mixed_host_and_device_maps():
    import numpy as np
    import torch
    import cpvs_gb300 as cp
    with pytest.raises(ValueError, match="host arrays or all CUDA tensors"):
        cp.MinMaxHierarchy.create_batch([np.zeros((8, 8), np.float32), torch.zeros((8, 8), device="cuda")])


def test_every_entry_point_refuses_null_handles(lib):
    """Every entry point called with null handles and pointers (sizes 1)
    returns CPVS_ERR_INVALID_ARG, or a neutral value for the queries, without
    touching the device."""
    import ctypes as C
    import cpvs_gb300
    not_status = {"cpvs_abi_version", "cpvs_shadow_uses_leafmasks", "cpvs_shadow_total_visibility",
                  "cpvs_ctx_get_option"}
    called = 0
    for name, (res, args) in sorted(cpvs_gb300._SIGS.items()):
        if res is C.c_char_p:
            continue
        vals = [None if (a is C.c_void_p or (isinstance(a, type) and issubclass(a, C._Pointer)))
                else (0.0 if a is C.c_float else 1) for a in args]
        r = getattr(lib, name)(*vals)
        called += 1
        if res is C.c_int and name not in not_status:
            assert r == 1, (name, r, lib.cpvs_last_error())
        elif name == "cpvs_shadow_total_visibility":
            assert r == 2
        elif name == "cpvs_ctx_get_option":
            assert r == -1
        elif res is not None and name != "cpvs_abi_version":
            assert not r, (name, r)  # sizes and counts of nothing are 0, handles null
    assert called >= 50


def test_header_is_plain_c(lib, tmp_path):
    """include/cpvs.h compiles as strict C99 and links from C; without a GPU
    the context call reports the device error (no fallback) and the program
    still exits cleanly."""
    import shutil
    import torch
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    src = tmp_path / "abi.c"
    src.write_text(
        '#include "cpvs.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        "    cpvs_ctx* ctx = NULL;\n"
        "    cpvs_build_job job = {0, 0, 1};\n"
        "    cpvs_server_config cfg = {0, 0, 0, CPVS_FLAG_LEAFMASKS};\n"
        "    cpvs_status s = cpvs_ctx_create(0, &ctx);\n"
        "    (void)job; (void)cfg;\n"
        '    if (s != CPVS_OK) { printf("%s\\n", cpvs_status_string(s)); return 0; }\n'
        '    printf("ok\\n");\n'
        "    cpvs_ctx_destroy(ctx);\n"
        "    return 0;\n"
        "}\n")
    libdir = os.path.join(ROOT, "cpvs_gb300")
    exe = str(tmp_path / "abi")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lcpvs_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120, check=True).stdout.strip()
    assert out == ("ok" if torch.cuda.is_available() else "CUDA device error")


def test_product_never_uses_the_oracle(lib):
    """The library links nothing of oracle/ and the package imports nothing
    from it: the oracle is test infrastructure only."""
    from cpvs_gb300 import LIB_PATH
    needed = subprocess.run(["readelf", "-d", LIB_PATH], capture_output=True, text=True, check=True).stdout
    assert "oracle" not in needed and "cpvs_ref" not in needed
    pkg = os.path.join(ROOT, "cpvs_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".hpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"^\s*(import oracle|from oracle)", src, re.M), f
                assert not re.search(r'#include\s*[<"][^>"]*oracle', src), f
    for f in os.listdir(os.path.join(ROOT, "include")):
        assert "oracle" not in open(os.path.join(ROOT, "include", f)).read(), f
