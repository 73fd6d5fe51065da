"""The saved form of shadows and grids, in plain numpy: the same bytes that
cpvs_shadow_serialize / cpvs_grid_serialize write and the *_deserialize
calls accept (layout in include/cpvs.h).  Lets tools inspect or produce DAG
files without a GPU."""
import struct

import numpy as np

MAGIC = b"CPVSDAG\0"
VERSION = 1
KIND_SHADOW, KIND_GRID = 0, 1
HEADER = struct.Struct("<8s6I2Q")  # magic, version, kind, numLevels, flags, length, reserved, words, checksum
assert HEADER.size == 48


def fnv1a64(data: bytes) -> int:
    """FNV-1a, 64-bit (offset basis 0xcbf29ce484222325, prime 0x100000001b3)."""
    a = np.frombuffer(data, np.uint8)
    h = 0xCBF29CE484222325
    prime, mask = 0x100000001B3, (1 << 64) - 1
    # byte-serial by definition; chunked through Python ints
    for b in a.tobytes():
        h = ((h ^ b) * prime) & mask
    return h


def _pack(kind, num_levels, leafmasks, length, words, body: bytes) -> bytes:
    return HEADER.pack(MAGIC, VERSION, kind, num_levels, 1 if leafmasks else 0, length, 0, words,
                       fnv1a64(body)) + body


def pack_shadow(dag, num_levels: int, leafmasks: bool, tree_nodes, unique_nodes) -> bytes:
    dag = np.ascontiguousarray(dag, "<u4")
    counts = np.zeros(2 * num_levels, "<u8")
    counts[:len(tree_nodes)] = tree_nodes
    counts[num_levels:num_levels + len(unique_nodes)] = unique_nodes
    return _pack(KIND_SHADOW, num_levels, leafmasks, 1, dag.size, counts.tobytes() + dag.tobytes())


def pack_grid(dag, cells, length: int, dag_levels: int, leafmasks: bool) -> bytes:
    dag = np.ascontiguousarray(dag, "<u4")
    cells = np.ascontiguousarray(cells, "<u4")
    assert cells.size == length ** 3
    return _pack(KIND_GRID, dag_levels, leafmasks, length, dag.size, cells.tobytes() + dag.tobytes())


def unpack(data: bytes) -> dict:
    """Parses and checks a saved shadow or grid; raises ValueError."""
    if len(data) < HEADER.size:
        raise ValueError("shorter than the header")
    magic, version, kind, nl, flags, length, reserved, words, checksum = HEADER.unpack_from(data)
    if magic != MAGIC or version != VERSION or kind not in (KIND_SHADOW, KIND_GRID) or reserved:
        raise ValueError("bad header")
    if kind == KIND_SHADOW:
        size = HEADER.size + 16 * nl + 4 * words
    else:
        size = HEADER.size + 4 * length ** 3 + 4 * words
    if len(data) < size:
        raise ValueError("truncated")
    body = data[HEADER.size:size]
    if fnv1a64(body) != checksum:
        raise ValueError("checksum mismatch")
    out = {"kind": kind, "num_levels": nl, "leafmasks": bool(flags & 1), "length": length}
    if kind == KIND_SHADOW:
        counts = np.frombuffer(body, "<u8", 2 * nl)
        out["tree_nodes"], out["unique_nodes"] = counts[:nl].tolist(), counts[nl:].tolist()
        out["dag"] = np.frombuffer(body, "<u4", words, 16 * nl).copy()
    else:
        out["cells"] = np.frombuffer(body, "<u4", length ** 3).copy()
        out["dag"] = np.frombuffer(body, "<u4", words, 4 * length ** 3).copy()
    return out
