"""CPU tests of the product's host side: the C ABI's symbol table and the reference formats."""
import ctypes
import os
import re
import struct

import numpy as np
import pytest

from conftest import REPO


def header_functions():
    """Every tdag_* function declared by the C headers (include/tdag.h, tdag_diag.h, tdag16.h, tdag_nn.h)."""
    names = set()
    for h in ("tdag.h", "tdag_diag.h", "tdag16.h", "tdag_nn.h"):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(tdag(?:16)?_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol(tdaglib):
    lib = ctypes.CDLL(tdaglib.library_path())
    names = header_functions()
    assert names, "no functions parsed from include/*.h"
    for n in names:
        assert hasattr(lib, n), f"libtdag.so does not export {n}"
    from tdag import _abi
    assert set(_abi.EXPORTED) == set(names)


def test_version_string(tdaglib):
    assert b"sm_103a" in tdaglib.lib().tdag_version()


def test_context_without_gpu_fails_loudly(tdaglib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tdaglib.TDagError) as ei:
        tdaglib.Context(0)
    assert ei.value.code == 7  # TDAG_ERR_NO_DEVICE


def test_config_bytes_layout(tdaglib):
    c = tdaglib.TransformDAGConfig(True, False, True, 4)
    b = c.to_bytes()
    assert len(b) == 8 and b[:4] == b"\x01\x00\x01\x00" and struct.unpack("<I", b[4:])[0] == 4
    assert tdaglib.TransformDAGConfig.from_bytes(b) == c


def test_tdag_format_roundtrip(oracle, tdaglib):
    from helpers import blocky_grid, dag_svo_bytes
    svo = dag_svo_bytes(oracle, blocky_grid(32, 4))
    ref, _, _ = oracle.construct_tdag(svo)
    s, cfg = tdaglib.read_tdag(ref)
    assert cfg == tdaglib.TransformDAGConfig()
    assert tdaglib.write_tdag(s, cfg) == ref


def test_corrupt_svo_rejected(tdaglib):
    with pytest.raises(tdaglib.TDagError):
        tdaglib.EditStructure.from_svo_bytes(b"\x00" * 4)
    with pytest.raises(tdaglib.TDagError):
        tdaglib.EditStructure.from_svo_bytes(struct.pack("<II", 72198382, 2) + struct.pack("<Q", 3))


def test_tp_sentinel_layout(tdaglib):
    # create(0xFFFFFFFF): identity permutation (0,1,2) and translations biased by 32
    v = tdaglib.TP_SENTINEL
    assert v & ((1 << 37) - 1) == 0xFFFFFFFF
    assert (v >> 40) & 63 == (0 | 1 << 2 | 2 << 4)
    assert all(((v >> (46 + 6 * k)) & 63) == 32 for k in range(3))


def test_voxel_count(oracle, tdaglib):
    from helpers import blocky_grid
    d = blocky_grid(32, 8)
    s = tdaglib.EditStructure.from_svo_bytes(oracle.to_dag(oracle.svo_from_dense(d)))
    assert s.compute_voxel_count() == int(d.sum())


def test_nn_entry_points_reject_bad_arguments_without_a_device(tdaglib):
    """The learned-proposal kernels' entry points validate their arguments before touching a device."""
    import ctypes as C
    from tdag import _abi
    L = tdaglib.lib()
    op = _abi.NnOperand(None, _abi.NN_KMAJOR, 0)
    assert L.tdag_nn_gemm(None, C.byref(op), C.byref(op), 1, 1, 16, 1.0, None, 0, None, 0, None, 1, 0) == _abi.TDAG_ERR_ARG
    assert L.tdag_nn_topk(None, None, 0, 8, None, None) == _abi.TDAG_ERR_ARG
    assert L.tdag_nn_block_masks(None, None, 0, 4, None) == _abi.TDAG_ERR_ARG
    assert L.tdag_nn_adamw(None, None, None, None, None, 0, 1e-3, 0.9, 0.999, 1e-8, 0.0, 1, None) == _abi.TDAG_ERR_ARG
    assert L.tdag_nn_info_nce(None, None, 0, None, None) == _abi.TDAG_ERR_ARG
    assert L.tdag_nn_sync(None) == _abi.TDAG_ERR_ARG


def test_batch_graph_entry_points_reject_bad_arguments_without_a_device(tdaglib):
    """tdag_batch_graph_*: null arguments and an empty batch are refused before any CUDA call, and
    freeing a null graph is a no-op."""
    import ctypes
    from tdag import _abi
    L = tdaglib.lib()
    out = ctypes.c_void_p()
    cfg = tdaglib._config_struct(tdaglib.TransformDAGConfig())
    views = (_abi.SvdagView * 1)()
    assert L.tdag_batch_graph_create(None, views, 1, ctypes.byref(cfg), ctypes.byref(out)) == _abi.TDAG_ERR_ARG
    assert L.tdag_batch_graph_create(None, views, 0, ctypes.byref(cfg), ctypes.byref(out)) == _abi.TDAG_ERR_ARG
    res = (ctypes.POINTER(_abi.Result) * 1)()
    assert L.tdag_batch_graph_launch(None, res, None) == _abi.TDAG_ERR_ARG
    assert L.tdag_batch_graph_free(None) == _abi.TDAG_OK


def test_checkpointed_scene_rejects_bad_arguments_without_a_device(tdaglib):
    import ctypes
    from tdag import _abi
    L = tdaglib.lib()
    out = ctypes.c_void_p()
    sc = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=256, chunk_resolution=64).to_c()
    assert L.tdag_scene_svdag_checkpointed(None, ctypes.byref(sc), b"x.ckpt", 1, 0, ctypes.byref(out)) == _abi.TDAG_ERR_ARG
    assert L.tdag_scene_svdag_checkpointed(None, ctypes.byref(sc), None, 1, 0, ctypes.byref(out)) == _abi.TDAG_ERR_ARG
