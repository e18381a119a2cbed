"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle (``tdag_oracle.cpp``) is a from-scratch CPU restatement of the reference's
Transform-DAG construction path. Only the test-suite, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg / reference arm may import this module; the product library
(``libtdag.so``) never links or calls it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    sources = [os.path.join(_HERE, f) for f in ("tdag_oracle.cpp", "tdag16_oracle.cpp", "scene_oracle.cpp", "Makefile")]
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(f) for f in sources)
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        u8pp = ctypes.POINTER(u8p)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_svo_from_dense.argtypes = [u8p, ctypes.c_uint32, u8pp, u64p]
        L.orc_to_dag.argtypes = [u8p, ctypes.c_uint64, u8pp, u64p]
        L.orc_construct_tdag.argtypes = [u8p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_uint32, u8pp, u64p, u64p, u64p]
        L.orc_find_duplicates.argtypes = [ctypes.c_uint32, u64p, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, u64p, u32p, u32p, u64p]
        L.orc_hierarchical.argtypes = [u8p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, u8pp, u64p]
        L.orc_tdag_decode.argtypes = [u8p, ctypes.c_uint64, u8p, ctypes.c_uint32]
        L.orc_transform_tables.argtypes = [u8p, u8p, u8p]
        L.orc_encode_fixed64.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
        L.orc_encode_fixed64.restype = ctypes.c_uint64
        L.orc_decode_fixed64.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
        L.orc_decode_fixed64.restype = ctypes.c_uint64
        L.orc16_last_error.restype = ctypes.c_char_p
        L.orc16_huffman_lengths.argtypes = [u64p, ctypes.c_uint32, ctypes.c_uint32, u32p]
        L.orc16_huffman_codes.argtypes = [u32p, ctypes.c_uint32, ctypes.c_int, u64p, u32p]
        L.orc16_huffman_decode.argtypes = [u64p, u32p, ctypes.c_uint32, ctypes.c_uint32, u32p, u32p]
        L.orc16_encode.argtypes = [u8p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, u8pp, u64p, u64p,
                                   ctypes.c_uint32]
        L.orc16_decode_dense.argtypes = [u8p, ctypes.c_uint64, u8p, ctypes.c_uint32]
        L.orc16_raycast.argtypes = [u8p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64,
                                    ctypes.POINTER(ctypes.c_float), u32p, u8p]
        L.orc_to_static.argtypes = [u8p, ctypes.c_uint64, u8pp, u64p]
        L.orc_construct_static_tdag.argtypes = [u8p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                                                u8pp, u64p]
        L.orc_static_tdag_decode.argtypes = [u8p, ctypes.c_uint64, u8p, ctypes.c_uint32]
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_scene_last_error.restype = ctypes.c_char_p
        L.orc_scene_primitives.argtypes = [ctypes.c_uint32] * 4 + [ctypes.c_void_p, ctypes.c_uint32, u32p]
        L.orc_scene_dense.argtypes = [ctypes.c_uint32] * 4 + [ctypes.c_int] + [ctypes.c_uint32] * 4 + [u8p]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _u8(buf: bytes):
    a = np.frombuffer(buf, dtype=np.uint8)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _take(out, n) -> bytes:
    try:
        return ctypes.string_at(out, n.value)
    finally:
        lib().orc_free(out)


def _chk(rc):
    if rc != 0:
        raise OracleError(lib().orc_last_error().decode())


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def svo_from_dense(dense: np.ndarray) -> bytes:
    """A1: EditStructure(VoxelGrid) -> .svo bytes. ``dense[z, y, x]`` (x fastest), bool/uint8."""
    d = np.ascontiguousarray(dense, dtype=np.uint8)
    res = d.shape[0]
    assert d.shape == (res, res, res)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    _chk(lib().orc_svo_from_dense(d.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), res, ctypes.byref(out), ctypes.byref(n)))
    return _take(out, n)


def to_dag(svo: bytes) -> bytes:
    """A2: EditStructure::toDAG on .svo bytes."""
    a, p = _u8(svo)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    _chk(lib().orc_to_dag(p, len(svo), ctypes.byref(out), ctypes.byref(n)))
    return _take(out, n)


STAT_KEYS = ("items", "probes", "hits", "candidates", "verifications", "verified", "table_entries", "unique")


def construct_tdag(svo: bytes, symmetry=True, axis=True, translation=True, max_level=4):
    """A6: constructTransformDAG -> (.tdag bytes incl. trailing config, stats dict, times_ns)."""
    a, p = _u8(svo)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    st = (ctypes.c_uint64 * 8)()
    tm = (ctypes.c_uint64 * 4)()
    _chk(lib().orc_construct_tdag(p, len(svo), int(symmetry), int(axis), int(translation), int(max_level),
                                  ctypes.byref(out), ctypes.byref(n), st, tm))
    return _take(out, n), dict(zip(STAT_KEYS, list(st))), list(tm)


def hierarchical(svo: bytes, symmetry=True, axis=True) -> bytes:
    a, p = _u8(svo)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    _chk(lib().orc_hierarchical(p, len(svo), int(symmetry), int(axis), ctypes.byref(out), ctypes.byref(n)))
    return _take(out, n)


def find_duplicates(level: int, grids: np.ndarray, symmetry=True, axis=True, translation=True):
    """Inner seam findDuplicatesAmongFlattenedItems_cpp2<level> on dense grids (n x W uint64)."""
    g = np.ascontiguousarray(grids, dtype=np.uint64)
    n = g.shape[0]
    mapping = np.zeros(n, dtype=np.uint64)
    uniq = np.zeros(max(n, 1), dtype=np.uint32)
    nu = ctypes.c_uint32()
    st = (ctypes.c_uint64 * 8)()
    _chk(lib().orc_find_duplicates(level, g.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n, int(symmetry), int(axis),
                                   int(translation), mapping.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                   uniq.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(nu), st))
    return mapping, uniq[: nu.value].copy(), dict(zip(STAT_KEYS, list(st)))


def tdag_decode(tdag: bytes, res: int) -> np.ndarray:
    a, p = _u8(tdag)
    dense = np.zeros((res, res, res), dtype=np.uint8)
    _chk(lib().orc_tdag_decode(p, len(tdag), dense.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), res))
    return dense


def transform_tables():
    c = np.zeros((48, 48), np.uint8)
    i = np.zeros(48, np.uint8)
    p = np.zeros((48, 8), np.uint8)
    f = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    lib().orc_transform_tables(f(c), f(i), f(p))
    return c, i, p


def encode_fixed64(tp: int, level: int) -> int:
    return int(lib().orc_encode_fixed64(tp, level))


def decode_fixed64(e: int, level: int) -> int:
    return int(lib().orc_decode_fixed64(e, level))


# ------------------------------------------------------------------------------------------------
# .tdag16 (tdag16_oracle.cpp)
# ------------------------------------------------------------------------------------------------
TIE_CANONICAL = 0  # ties by ascending item index / ascending pointer value (the library's canonical option)
TIE_LIBSTDCXX = 1  # std::sort + std::unordered_map, as the reference behaves with libstdc++ (serial backend)
LEVEL16_KEYS = ("num_nodes", "memory_in_bytes", "table_size", "unique_pointers", "table_u16", "table_u32",
                "table_u48", "direct_u16", "direct_u32", "direct_u48")


def _chk16(rc):
    if rc != 0:
        raise OracleError(lib().orc16_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def huffman_lengths(freq, max_len):
    f = np.ascontiguousarray(freq, dtype=np.uint64)
    out = np.zeros(len(f), np.uint32)
    _chk16(lib().orc16_huffman_lengths(_p(f, ctypes.c_uint64), len(f), max_len, _p(out, ctypes.c_uint32)))
    return [int(v) for v in out]


def huffman_codes(lengths, lsb=False):
    l = np.ascontiguousarray(lengths, dtype=np.uint32)
    codes = np.zeros(len(l), np.uint64)
    bits = np.zeros(len(l), np.uint32)
    _chk16(lib().orc16_huffman_codes(_p(l, ctypes.c_uint32), len(l), int(lsb), _p(codes, ctypes.c_uint64),
                                     _p(bits, ctypes.c_uint32)))
    return [(int(c), int(b)) for c, b in zip(codes, bits)]


def huffman_decode(codes, key):
    c = np.array([x for x, _ in codes], np.uint64)
    b = np.array([y for _, y in codes], np.uint32)
    s, n = ctypes.c_uint32(), ctypes.c_uint32()
    _chk16(lib().orc16_huffman_decode(_p(c, ctypes.c_uint64), _p(b, ctypes.c_uint32), len(c), key, ctypes.byref(s),
                                      ctypes.byref(n)))
    return int(s.value), int(n.value)


def encode_tdag16(tdag: bytes, pointer_tables=False, huffman=False, tie=TIE_LIBSTDCXX):
    """constructTransformDAG16 on .tdag bytes -> (.tdag16 bytes, per-level stats dicts). The default tie
    order is the reference's (libstdc++), which the reference compiled here reproduces byte for byte."""
    a, p = _u8(tdag)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    st = np.zeros((32, 10), np.uint64)
    _chk16(lib().orc16_encode(p, len(tdag), int(pointer_tables), int(huffman), int(tie), ctypes.byref(out),
                              ctypes.byref(n), _p(st, ctypes.c_uint64), 32))
    data = _take(out, n)
    root = int.from_bytes(tdag[-16:-12], "little")  # ..., resolution, rootLevel, structureType, config(8)
    return data, [dict(zip(LEVEL16_KEYS, (int(v) for v in st[l]))) for l in range(root + 1)]


def decode_tdag16(data: bytes, res: int) -> np.ndarray:
    """Every voxel of a .tdag16, as dense[z, y, x]."""
    a, p = _u8(data)
    dense = np.zeros((res, res, res), dtype=np.uint8)
    _chk16(lib().orc16_decode_dense(p, len(data), _p(dense, ctypes.c_uint8), res))
    return dense


def raycast_tdag16(data: bytes, rays: np.ndarray):
    """First solid voxel per ray (n x 8 float32: origin, direction, tmin, tmax) by voxel DDA over the
    decoder, double precision -> (t float32 [n], voxel uint32 [n, 3], hit uint8 [n])."""
    a, p = _u8(data)
    r = np.ascontiguousarray(rays, dtype=np.float32)
    n = r.shape[0]
    t = np.zeros(n, np.float32)
    vox = np.zeros((n, 3), np.uint32)
    hit = np.zeros(n, np.uint8)
    _chk16(lib().orc16_raycast(p, len(data), _p(r, ctypes.c_float), n, _p(t, ctypes.c_float), _p(vox, ctypes.c_uint32),
                               _p(hit, ctypes.c_uint8)))
    return t, vox, hit


# ------------------------------------------------------------------------------------------------
# StaticStructure path (constructStaticTransformDAG)
# ------------------------------------------------------------------------------------------------
def to_static(svo: bytes) -> bytes:
    """StaticStructure<void, uint32_t>(EditStructure) of an .svo, as StaticStructure::writeTo bytes."""
    a, p = _u8(svo)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    _chk(lib().orc_to_static(p, len(svo), ctypes.byref(out), ctypes.byref(n)))
    return _take(out, n)


def construct_static_tdag(static_bytes: bytes, symmetry=True, axis=True, translation=True, max_level=4) -> bytes:
    """constructStaticTransformDAG -> StaticStructure<void, TransformPointer>::writeTo bytes."""
    a, p = _u8(static_bytes)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    _chk(lib().orc_construct_static_tdag(p, len(static_bytes), int(symmetry), int(axis), int(translation), int(max_level),
                                         ctypes.byref(out), ctypes.byref(n)))
    return _take(out, n)


def static_tdag_decode(static_tdag: bytes, res: int) -> np.ndarray:
    a, p = _u8(static_tdag)
    dense = np.zeros((res, res, res), dtype=np.uint8)
    _chk(lib().orc_static_tdag_decode(p, len(static_tdag), dense.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), res))
    return dense


# ------------------------------------------------------------------------------------------------
# Procedural primitive scenes (scene_oracle.cpp)
# ------------------------------------------------------------------------------------------------
PRIMITIVE_DTYPE = np.dtype([("type", "<u4"), ("xform", "<u4"), ("size", "<i4", 3), ("radius", "<i4"), ("offset", "<i4", 3),
                            ("seed", "<u4"), ("source", "<u4"), ("reserved", "<u4")])


def scene_primitives(resolution: int, seed: int, num_primitives: int, copy_percent: int = 30) -> np.ndarray:
    """The primitive list of a scene, as a structured array laid out like tdag_primitive."""
    out = np.zeros(max(num_primitives, 1), PRIMITIVE_DTYPE)
    n = ctypes.c_uint32()
    if lib().orc_scene_primitives(resolution, seed, num_primitives, copy_percent, out.ctypes.data_as(ctypes.c_void_p), len(out),
                                  ctypes.byref(n)) != 0:
        raise OracleError(lib().orc_scene_last_error().decode())
    return out[: n.value]


def scene_dense(resolution: int, seed: int, num_primitives: int, copy_percent: int = 30, shell: bool = True, origin=(0, 0, 0),
                size: int = 0) -> np.ndarray:
    """dense[z, y, x] of the sub-box of side ``size`` (default: the whole grid) at ``origin`` of a
    primitive scene: exactly the restriction of the whole grid, its shell included."""
    size = size or resolution
    dense = np.zeros((size, size, size), np.uint8)
    if lib().orc_scene_dense(resolution, seed, num_primitives, copy_percent, int(shell), int(origin[0]), int(origin[1]), int(origin[2]),
                             size, dense.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))) != 0:
        raise OracleError(lib().orc_scene_last_error().decode())
    return dense
