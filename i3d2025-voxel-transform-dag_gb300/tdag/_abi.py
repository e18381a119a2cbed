"""ctypes declarations of the C ABI in include/tdag.h (libtdag.so)."""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
_LIB_FILE = os.path.join(PKG, "build", "libtdag.so")

TDAG_OK = 0
TDAG_ERR_ARG = 1
TDAG_ERR_OOM = 2
TDAG_ERR_TABLE_FULL = 3
TDAG_ERR_ALLOC = 4
TDAG_ERR_CUDA = 5
TDAG_ERR_CORRUPT = 6
TDAG_ERR_NO_DEVICE = 7
TDAG_ERR_INTERRUPTED = 8
MAX_LEVELS = 32

ERROR_NAMES = {1: "ARG", 2: "OOM", 3: "TABLE_FULL", 4: "ALLOC", 5: "CUDA", 6: "CORRUPT", 7: "NO_DEVICE", 8: "INTERRUPTED"}


class TDagError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"tdag error {code} ({ERROR_NAMES.get(code, '?')}): {message}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("symmetry", ctypes.c_int32), ("axis_permutation", ctypes.c_int32),
                ("translation", ctypes.c_int32), ("max_translation_level", ctypes.c_uint32)]


class SvdagView(ctypes.Structure):
    _fields_ = [("resolution", ctypes.c_uint32), ("root_level", ctypes.c_uint32),
                ("structure_type", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("nodes", ctypes.POINTER(ctypes.c_uint32) * MAX_LEVELS),
                ("node_counts", ctypes.c_uint64 * MAX_LEVELS),
                ("leaves", ctypes.POINTER(ctypes.c_uint64)), ("leaf_count", ctypes.c_uint64)]


class LevelStats(ctypes.Structure):
    _fields_ = [("items", ctypes.c_uint64), ("unique", ctypes.c_uint64), ("probes", ctypes.c_uint64),
                ("filter_pass", ctypes.c_uint64), ("hits", ctypes.c_uint64), ("candidates", ctypes.c_uint64),
                ("verifications", ctypes.c_uint64), ("verified", ctypes.c_uint64),
                ("table_entries", ctypes.c_uint64), ("search_ms", ctypes.c_float), ("probe_ms", ctypes.c_float)]


class Stats(ctypes.Structure):
    _fields_ = [("hierarchical", LevelStats * MAX_LEVELS), ("translation", LevelStats * MAX_LEVELS),
                ("total_ms", ctypes.c_float), ("hierarchical_ms", ctypes.c_float),
                ("translation_ms", ctypes.c_float), ("table_regrows", ctypes.c_uint32), ("kernel_launches", ctypes.c_uint64)]


class Result(ctypes.Structure):
    _fields_ = [("resolution", ctypes.c_uint32), ("root_level", ctypes.c_uint32),
                ("structure_type", ctypes.c_uint32), ("on_device", ctypes.c_uint32),
                ("nodes", ctypes.POINTER(ctypes.c_uint64) * MAX_LEVELS),
                ("node_counts", ctypes.c_uint64 * MAX_LEVELS),
                ("leaves", ctypes.POINTER(ctypes.c_uint64)), ("leaf_count", ctypes.c_uint64),
                ("stats", Stats)]


class StaticView(ctypes.Structure):
    _fields_ = [("resolution", ctypes.c_uint32), ("root_level", ctypes.c_uint32),
                ("structure_type", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("words", ctypes.POINTER(ctypes.c_uint32) * MAX_LEVELS),
                ("word_counts", ctypes.c_uint64 * MAX_LEVELS),
                ("leaves", ctypes.POINTER(ctypes.c_uint64)), ("leaf_count", ctypes.c_uint64)]


class StaticResult(ctypes.Structure):
    _fields_ = [("resolution", ctypes.c_uint32), ("root_level", ctypes.c_uint32),
                ("structure_type", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("words", ctypes.POINTER(ctypes.c_uint64) * MAX_LEVELS),
                ("word_counts", ctypes.c_uint64 * MAX_LEVELS),
                ("leaves", ctypes.POINTER(ctypes.c_uint64)), ("leaf_count", ctypes.c_uint64),
                ("stats", Stats)]


class Scene(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("resolution", ctypes.c_uint32), ("seed", ctypes.c_uint32),
                ("num_primitives", ctypes.c_uint32), ("copy_percent", ctypes.c_uint32), ("shell", ctypes.c_uint32),
                ("chunk_resolution", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Primitive(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("xform", ctypes.c_uint32), ("size", ctypes.c_int32 * 3),
                ("radius", ctypes.c_int32), ("offset", ctypes.c_int32 * 3), ("seed", ctypes.c_uint32),
                ("source", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Tuning(ctypes.Structure):
    _fields_ = [("filter_bits_per_key", ctypes.c_uint32), ("table_load_percent", ctypes.c_uint32),
                ("search_ctas_per_sm", ctypes.c_uint32), ("class_table_load_percent", ctypes.c_uint32),
                ("table_regrow_limit", ctypes.c_uint32), ("slab_pool_slabs", ctypes.c_uint32), ("device_memory_limit", ctypes.c_uint64),
                ("probe_bulk_copy", ctypes.c_uint32), ("verify_lanes", ctypes.c_uint32), ("lookup_tile", ctypes.c_uint32),
                ("reserved3", ctypes.c_uint32)]


class EncodingConfig(ctypes.Structure):
    _fields_ = [("pointer_tables", ctypes.c_int32), ("huffman_code", ctypes.c_int32), ("tie_order", ctypes.c_int32)]


class Tdag16LevelStats(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_uint64), ("memory_in_bytes", ctypes.c_uint64), ("table_size", ctypes.c_uint64),
                ("unique_pointers", ctypes.c_uint64), ("table_pointers", ctypes.c_uint64 * 3),
                ("direct_pointers", ctypes.c_uint64 * 3)]


class Tdag16Result(ctypes.Structure):
    _fields_ = [("bytes", ctypes.POINTER(ctypes.c_uint8)), ("size", ctypes.c_uint64), ("root_level", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("levels", Tdag16LevelStats * MAX_LEVELS), ("encode_ms", ctypes.c_float),
                ("wall_ms", ctypes.c_float), ("kernel_launches", ctypes.c_uint64)]


class Tdag16VerifyStats(ctypes.Structure):
    _fields_ = [("existence_mismatches", ctypes.c_uint64), ("voxel_mismatches", ctypes.c_uint64),
                ("boxes_compared", ctypes.c_uint64), ("pairs_walked", ctypes.c_uint64), ("box_level", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


# Every symbol include/tdag.h declares (checked by the CPU test-suite).
EXPORTED = (
    "tdag_version", "tdag_last_error_message", "tdag_ctx_create", "tdag_ctx_destroy", "tdag_ctx_stream",
    "tdag_build", "tdag_build_device", "tdag_result_free", "tdag_find_duplicates_level", "tdag_build_hierarchical",
    "tdag_scene_primitives", "tdag_scene_svdag", "tdag_svdag_from_dense", "tdag_svdag_get_view", "tdag_svdag_voxel_count",
    "tdag_svdag_copy_level", "tdag_svdag_free", "tdag_find_duplicates_level_noalloc", "tdag_scene_svdag_checkpointed",
    "tdag_build_batched", "tdag_build_batched_device", "tdag_result_to_host",
    "tdag_find_duplicates_level_device", "tdag_build_device_proposed", "tdag_device_copy",
    "tdag_build_static", "tdag_static_result_free",
    "tdag_batch_graph_create", "tdag_batch_graph_launch", "tdag_batch_graph_free",
    "tdag_l2_probe_peak",  # include/tdag_diag.h
    "tdag_device_pool_usage",  # include/tdag_diag.h
    "tdag_encode16", "tdag16_result_free", "tdag16_huffman_code_table",  # include/tdag16.h
    "tdag16_upload", "tdag16_device_free", "tdag16_get", "tdag16_verify", "tdag16_raycast",
    "tdag_nn_gemm", "tdag_nn_block_masks", "tdag_nn_pool_forward", "tdag_nn_pool_backward",  # include/tdag_nn.h
    "tdag_nn_info_nce", "tdag_nn_column_sums", "tdag_nn_adamw", "tdag_nn_topk", "tdag_nn_sync", "tdag_nn_to_bf16",
    "tdag_nn_canon_gather", "tdag_nn_canon_scatter",
)

# include/tdag_nn.h operand modes
NN_KMAJOR, NN_MNMAJOR, NN_BITS, NN_BITS_T = 0, 1, 2, 3


class NnOperand(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("mode", ctypes.c_uint32), ("ld", ctypes.c_uint32)]

# int (*tdag_proposal_fn)(void* user, uint32_t level, const uint64_t* d_grids, uint32_t n, uint32_t* d_sources, uint32_t* num_sources)
PROPOSAL_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                               ctypes.POINTER(ctypes.c_uint32))

_lib = None


def library_path() -> str:
    return _LIB_FILE


def lib(path: str = None):
    """Load libtdag.so. Raises TDagError if it has not been built (no fallback path exists)."""
    global _lib
    if _lib is None:
        p = path or _LIB_FILE
        if not os.path.exists(p):
            raise TDagError(TDAG_ERR_NO_DEVICE, f"libtdag.so not built at {p}; run build_lib.py (or __graft_entry__.build())")
        L = ctypes.CDLL(p)
        vp = ctypes.c_void_p
        L.tdag_version.restype = ctypes.c_char_p
        L.tdag_last_error_message.restype = ctypes.c_char_p
        L.tdag_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(Tuning), ctypes.POINTER(vp)]
        L.tdag_ctx_destroy.argtypes = [vp]
        L.tdag_ctx_stream.argtypes = [vp, ctypes.POINTER(vp)]
        L.tdag_build.argtypes = [vp, ctypes.POINTER(SvdagView), ctypes.POINTER(Config), ctypes.POINTER(ctypes.POINTER(Result))]
        L.tdag_build_device.argtypes = [vp, ctypes.POINTER(SvdagView), ctypes.POINTER(Config), ctypes.POINTER(ctypes.POINTER(Result))]
        L.tdag_build_hierarchical.argtypes = [vp, ctypes.POINTER(SvdagView), ctypes.POINTER(Config), ctypes.POINTER(ctypes.POINTER(Result))]
        L.tdag_result_free.argtypes = [ctypes.POINTER(Result)]
        L.tdag_find_duplicates_level.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32,
                                                 ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_uint64),
                                                 ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                                 ctypes.POINTER(LevelStats)]
        L.tdag_scene_primitives.argtypes = [ctypes.POINTER(Scene), ctypes.POINTER(Primitive), ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
        L.tdag_scene_svdag.argtypes = [vp, ctypes.POINTER(Scene), ctypes.c_int, ctypes.POINTER(vp)]
        L.tdag_scene_svdag_checkpointed.argtypes = [vp, ctypes.POINTER(Scene), ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(vp)]
        L.tdag_svdag_from_dense.argtypes = [vp, ctypes.POINTER(ctypes.c_uint8), ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(vp)]
        L.tdag_svdag_get_view.argtypes = [vp, ctypes.POINTER(SvdagView)]
        L.tdag_svdag_voxel_count.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
        L.tdag_svdag_copy_level.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint64]
        L.tdag_svdag_free.argtypes = [vp]
        L.tdag_find_duplicates_level_noalloc.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.POINTER(Config),
                                                         vp, vp, vp]
        L.tdag_result_to_host.argtypes = [vp, ctypes.POINTER(Result), ctypes.POINTER(ctypes.POINTER(Result))]
        L.tdag_l2_probe_peak.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]
        L.tdag_device_pool_usage.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        L.tdag_find_duplicates_level_device.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.POINTER(Config), vp, ctypes.c_uint32,
                                                        vp, vp, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(LevelStats)]
        L.tdag_build_device_proposed.argtypes = [vp, ctypes.POINTER(SvdagView), ctypes.POINTER(Config), PROPOSAL_FN, vp,
                                                 ctypes.POINTER(ctypes.POINTER(Result))]
        L.tdag_device_copy.argtypes = [vp, vp, vp, ctypes.c_uint64]
        L.tdag_build_static.argtypes = [vp, ctypes.POINTER(StaticView), ctypes.POINTER(Config), ctypes.POINTER(ctypes.POINTER(StaticResult))]
        L.tdag_static_result_free.argtypes = [ctypes.POINTER(StaticResult)]
        L.tdag_encode16.argtypes = [vp, ctypes.POINTER(Result), ctypes.POINTER(Config), ctypes.POINTER(EncodingConfig),
                                    ctypes.POINTER(ctypes.POINTER(Tdag16Result))]
        L.tdag16_result_free.argtypes = [ctypes.POINTER(Tdag16Result)]
        L.tdag16_upload.argtypes = [vp, ctypes.POINTER(ctypes.c_uint8), ctypes.c_uint64, ctypes.POINTER(vp)]
        L.tdag16_device_free.argtypes = [vp]
        L.tdag16_get.argtypes = [vp, vp, vp, ctypes.c_uint64, vp]
        L.tdag16_raycast.argtypes = [vp, vp, vp, ctypes.c_uint64, vp]
        L.tdag16_verify.argtypes = [vp, vp, ctypes.POINTER(SvdagView), ctypes.POINTER(Tdag16VerifyStats)]
        L.tdag16_huffman_code_table.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)]
        u32, f32 = ctypes.c_uint32, ctypes.c_float
        L.tdag_nn_gemm.argtypes = [vp, ctypes.POINTER(NnOperand), ctypes.POINTER(NnOperand), u32, u32, u32, f32, vp, ctypes.c_int, vp, u32,
                                   vp, u32, ctypes.c_int]
        L.tdag_nn_block_masks.argtypes = [vp, vp, u32, u32, vp]
        L.tdag_nn_pool_forward.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp]
        L.tdag_nn_pool_backward.argtypes = [vp, vp, vp, vp, vp, vp, u32, u32, vp]
        L.tdag_nn_info_nce.argtypes = [vp, vp, u32, vp, vp]
        L.tdag_nn_column_sums.argtypes = [vp, vp, u32, u32, u32, vp]
        L.tdag_nn_adamw.argtypes = [vp, vp, vp, vp, vp, ctypes.c_uint64, f32, f32, f32, f32, f32, u32, vp]
        L.tdag_nn_topk.argtypes = [vp, vp, u32, u32, vp, vp]
        L.tdag_nn_sync.argtypes = [vp]
        L.tdag_nn_to_bf16.argtypes = [vp, vp, ctypes.c_uint64, vp]
        L.tdag_nn_canon_gather.argtypes = [vp, vp, u32, vp, u32, vp, vp]
        L.tdag_nn_canon_scatter.argtypes = [vp, vp, ctypes.c_int, vp, vp, u32, vp, u32]
        for fn in (L.tdag_build_batched, L.tdag_build_batched_device):
            fn.argtypes = [vp, ctypes.POINTER(SvdagView), ctypes.c_uint32, ctypes.POINTER(Config),
                           ctypes.POINTER(ctypes.POINTER(Result)), ctypes.POINTER(Stats)]
        L.tdag_batch_graph_create.argtypes = [vp, ctypes.POINTER(SvdagView), ctypes.c_uint32, ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.tdag_batch_graph_launch.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(Result)), ctypes.POINTER(Stats)]
        L.tdag_batch_graph_free.argtypes = [vp]
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != TDAG_OK:
        raise TDagError(rc, lib().tdag_last_error_message().decode(errors="replace"))


def level_stats_to_dict(s: LevelStats) -> dict:
    return {k: getattr(s, k) for k, _ in LevelStats._fields_ if k != "reserved"}


def stats_to_dict(s: Stats, root_level: int) -> dict:
    return {
        "kernel_launches": s.kernel_launches, "total_ms": s.total_ms, "hierarchical_ms": s.hierarchical_ms, "translation_ms": s.translation_ms,
        "table_regrows": s.table_regrows,
        "hierarchical": {l: level_stats_to_dict(s.hierarchical[l]) for l in range(2, root_level + 1)},
        "translation": {l: level_stats_to_dict(s.translation[l]) for l in range(2, 5)},
    }
