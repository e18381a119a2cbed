"""ctypes binding of the reference's own Transform-DAG code, compiled into oracle/_ref (test infrastructure).

``oracle/ref.mk`` compiles the reference's sources where they lie, with the self-written stand-in
headers of ``oracle/ref_shim/`` for its third-party libraries, into ``oracle/_ref/libtdag_ref.so``.
It can be built only where the reference's sources are present. The test-suite uses it to pin the
CPU restatement (``oracle.py``) to the reference itself, and ``tests/golden/make_golden.py`` uses it
to write golden digests. The product never loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libtdag_ref.so")
REFERENCE_ROOT = os.environ.get("TDAG_REFERENCE_ROOT", "/root/reference")
_lib = None


def sources_present() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "tools", "lib", "src", "voxel", "find_translation.cpp"))


def build(force: bool = False) -> str | None:
    """Build oracle/_ref/libtdag_ref.so from the reference's sources; None where they are absent."""
    if not sources_present():
        return LIB_PATH if os.path.exists(LIB_PATH) else None
    args = ["make", "-s", f"-j{os.cpu_count() or 4}", "-C", _HERE, "-f", "ref.mk", f"REF={REFERENCE_ROOT}"]
    if force:
        args.append("-B")
    subprocess.run(args, check=True)
    return LIB_PATH


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            build()
        L = ctypes.CDLL(LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        u8pp = ctypes.POINTER(u8p)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        i = ctypes.c_int
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_free.argtypes = [ctypes.c_void_p]
        L.ref_svo_from_dense.argtypes = [u8p, ctypes.c_uint32, u8pp, u64p]
        L.ref_to_dag.argtypes = [u8p, ctypes.c_uint64, u8pp, u64p]
        L.ref_construct_tdag.argtypes = [u8p, ctypes.c_uint64, i, i, i, ctypes.c_uint32, u8pp, u64p]
        L.ref_hierarchical.argtypes = [u8p, ctypes.c_uint64, i, i, u8pp, u64p]
        L.ref_encode_tdag16.argtypes = [u8p, ctypes.c_uint64, i, i, u8pp, u64p]
        L.ref_to_static.argtypes = [u8p, ctypes.c_uint64, u8pp, u64p]
        L.ref_construct_static_tdag.argtypes = [u8p, ctypes.c_uint64, i, i, i, ctypes.c_uint32, u8pp, u64p]
        L.ref_encode_static_tdag16.argtypes = [u8p, ctypes.c_uint64, i, i, i, ctypes.c_uint32, i, i, u8pp, u64p]
        _lib = L
    return _lib


class ReferenceError_(RuntimeError):
    pass


def _call(fn, *args) -> bytes:
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_uint64()
    if fn(*args, ctypes.byref(out), ctypes.byref(n)) != 0:
        raise ReferenceError_(lib().ref_last_error().decode())
    try:
        return ctypes.string_at(out, n.value)
    finally:
        lib().ref_free(out)


def _buf(data: bytes):
    a = np.frombuffer(data, dtype=np.uint8)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(data)


def svo_from_dense(dense: np.ndarray) -> bytes:
    """EditStructure(VoxelGrid) of ``dense[z, y, x]``, as .svo bytes."""
    d = np.ascontiguousarray(dense, dtype=np.uint8)
    return _call(lib().ref_svo_from_dense, d.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), d.shape[0])


def to_dag(svo: bytes) -> bytes:
    return _call(lib().ref_to_dag, *_buf(svo))


def construct_tdag(svo: bytes, symmetry=True, axis=True, translation=True, max_level=4) -> bytes:
    """constructTransformDAG, as .tdag bytes (structure, then the 8-byte config)."""
    return _call(lib().ref_construct_tdag, *_buf(svo), int(symmetry), int(axis), int(translation), int(max_level))


def hierarchical(svo: bytes, symmetry=True, axis=True) -> bytes:
    return _call(lib().ref_hierarchical, *_buf(svo), int(symmetry), int(axis))


def encode_tdag16(tdag: bytes, pointer_tables=False, huffman=False) -> bytes:
    return _call(lib().ref_encode_tdag16, *_buf(tdag), int(pointer_tables), int(huffman))


def to_static(svo: bytes) -> bytes:
    return _call(lib().ref_to_static, *_buf(svo))


def construct_static_tdag(static_bytes: bytes, symmetry=True, axis=True, translation=True, max_level=4) -> bytes:
    return _call(lib().ref_construct_static_tdag, *_buf(static_bytes), int(symmetry), int(axis), int(translation),
                 int(max_level))


def encode_static_tdag16(static_tdag: bytes, symmetry=True, axis=True, translation=True, max_level=4, pointer_tables=False,
                         huffman=False) -> bytes:
    """constructTransformDAG16 of a StaticStructure<void, TransformPointer> (StaticStructure::writeTo bytes)."""
    return _call(lib().ref_encode_static_tdag16, *_buf(static_tdag), int(symmetry), int(axis), int(translation), int(max_level),
                 int(pointer_tables), int(huffman))
