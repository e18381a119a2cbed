"""Host-side mirror of the reference's Transform-DAG construction interface, on libtdag.so.

The names follow tools/lib/include/voxcom/voxel/transform_dag.h and structure.h:

* :class:`EditStructure` mirrors ``EditStructure<void, uint32_t>`` (structure.h:159-211) and
  ``EditStructure<void, TransformPointer>`` (``child_type="transform"``), with the reference's
  binary layout (``writeTo``/``readFrom``, structure.h:483-501) and the ``.svo`` wrapper
  (export_import_structure.cpp:12-45).
* :class:`TransformDAGConfig` mirrors ``TransformDAGConfig`` (transform_dag.h:157-160).
* :func:`construct_transform_dag` mirrors ``constructTransformDAG`` (transform_dag.h:161-162),
  :func:`construct_transform_dag_hierarchical` mirrors ``constructTransformDAGHierarchical``
  (transform_dag.h:168-169) and :func:`find_duplicates_among_flattened_items` mirrors
  ``findDuplicatesAmongFlattenedItems_cpp2`` (transform_dag.h:307-308).

Every computation runs in libtdag.so on the GPU. There is no CPU fallback: if the library is
missing or no CUDA device is present, the call raises :class:`TDagError`.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
import struct
from typing import List, Optional

import numpy as np

from . import _abi
from ._abi import TDagError, lib, library_path  # noqa: F401

SVO_MAGIC = 72198382
SVO_VERSION = 2
EMPTY_CHILD = 0xFFFFFFFF


# ------------------------------------------------------------------------------------------------
# TransformPointer (transform_dag.h:19-151)
# ------------------------------------------------------------------------------------------------
PERMUTATIONS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))
PTR_MASK = (1 << 37) - 1


def tp_create(ptr: int, symmetry=(False, False, False), axis_permutation=(0, 1, 2), translation=(0, 0, 0)) -> int:
    """TransformPointer::create (transform_dag.h:46-54) as a raw uint64."""
    v = ptr & PTR_MASK
    v |= (int(symmetry[0]) | int(symmetry[1]) << 1 | int(symmetry[2]) << 2) << 37
    v |= (axis_permutation[0] | axis_permutation[1] << 2 | axis_permutation[2] << 4) << 40
    for k in range(3):
        v |= ((translation[k] + 32) & 63) << (46 + 6 * k)
    return v


def tp_decode(v: int):
    """(ptr, symmetry bools, axis permutation, translation) of a raw TransformPointer."""
    v = int(v)
    sym = (v >> 37) & 7
    return (v & PTR_MASK, (bool(sym & 1), bool(sym & 2), bool(sym & 4)),
            ((v >> 40) & 3, (v >> 42) & 3, (v >> 44) & 3),
            tuple(((v >> (46 + 6 * k)) & 63) - 32 for k in range(3)))


TP_SENTINEL = tp_create(0xFFFFFFFF)


def encode_fixed64(v: int, level: int) -> int:
    """TransformPointer::encodeFixed64 (transform_dag.h:375-397)."""
    ptr, sym, perm, t = tp_decode(v)
    out = ptr
    out = (out << 3) | (2 * perm[0] + (1 if perm[2] < perm[1] else 0))
    out = (out << 3) | (int(sym[0]) | int(sym[1]) << 1 | int(sym[2]) << 2)
    if level:
        sb = level + 1
        for k in (2, 1, 0):
            out = (out << sb) | (t[k] + (1 << level))
    return out & 0xFFFFFFFFFFFFFFFF


@dataclasses.dataclass
class TransformDAGConfig:
    """TransformDAGConfig (transform_dag.h:157-160)."""

    symmetry: bool = True
    axis_permutation: bool = True
    translation: bool = True
    max_translation_level: int = 4

    def to_bytes(self) -> bytes:
        # three bools, one padding byte (written as zero), uint32
        return struct.pack("<???xI", self.symmetry, self.axis_permutation, self.translation, self.max_translation_level)

    @classmethod
    def from_bytes(cls, b: bytes) -> "TransformDAGConfig":
        s, a, t, m = struct.unpack("<???xI", b[:8])
        return cls(s, a, t, m)


@dataclasses.dataclass
class TransformEncodingConfig:
    """TransformEncodingConfig (tools/svdag_encoding/src/transform_dag_encoding.h:180-182). The
    svdag_encoding tool defaults both flags off (main.cpp:34); the renderer's files set both.

    ``tie_order`` is not a reference setting: "reference" (the default) gives the reference's bytes
    (equal reference counts ordered by libstdc++'s std::sort and std::unordered_map iteration, two
    host steps per level); "canonical" orders them by index and pointer value on the device only."""

    pointer_tables: bool = False
    huffman_code: bool = False
    tie_order: str = "reference"

    def tie_code(self) -> int:
        try:
            return {"reference": 0, "canonical": 1}[self.tie_order]
        except KeyError:
            raise ValueError(f"tie_order must be 'reference' or 'canonical', not {self.tie_order!r}") from None


# ------------------------------------------------------------------------------------------------
# EditStructure
# ------------------------------------------------------------------------------------------------
@dataclasses.dataclass
class EditStructure:
    """EditStructure<void, Child>. ``nodes_per_level[l]`` is an (n, 8) array: uint32 children
    (empty = 0xFFFFFFFF) for ``child_type="u32"``, uint64 TransformPointers for ``"transform"``.
    ``sub_grids`` holds the level-2 4x4x4 Morton bitmasks."""

    nodes_per_level: List[np.ndarray]
    sub_grids: np.ndarray
    resolution: int
    root_level: int
    structure_type: int = 0  # 0 = Tree, 1 = DAG
    child_type: str = "u32"

    SUB_GRID_LEVEL = 2

    @property
    def child_dtype(self):
        return np.uint32 if self.child_type == "u32" else np.uint64

    # ---- reference binary layout (BinaryWriter, binary_writer.h:48-78)
    def to_bytes(self) -> bytes:
        out = [struct.pack("<Q", len(self.nodes_per_level))]
        for lvl in self.nodes_per_level:
            a = np.ascontiguousarray(lvl, dtype=self.child_dtype).reshape(-1, 8)
            out.append(struct.pack("<Q", a.shape[0]))
            out.append(a.tobytes())
        sg = np.ascontiguousarray(self.sub_grids, dtype=np.uint64)
        out.append(struct.pack("<Q", sg.shape[0]))
        out.append(sg.tobytes())
        out.append(struct.pack("<III", self.resolution, self.root_level, self.structure_type))
        return b"".join(out)

    @classmethod
    def from_bytes(cls, buf: bytes, offset: int = 0, child_type: str = "u32"):
        """Parse a structure; returns (structure, offset after it)."""
        dt = np.uint32 if child_type == "u32" else np.uint64
        esz = 8 * np.dtype(dt).itemsize

        def take(n):
            nonlocal offset
            if offset + n > len(buf):
                raise TDagError(_abi.TDAG_ERR_CORRUPT, "truncated structure")
            b = buf[offset: offset + n]
            offset += n
            return b

        (nl,) = struct.unpack("<Q", take(8))
        if nl > 64:
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "corrupt level count")
        levels = []
        for _ in range(nl):
            (cnt,) = struct.unpack("<Q", take(8))
            levels.append(np.frombuffer(take(cnt * esz), dtype=dt).reshape(cnt, 8).copy())
        (cnt,) = struct.unpack("<Q", take(8))
        sg = np.frombuffer(take(cnt * 8), dtype=np.uint64).copy()
        res, root, st = struct.unpack("<III", take(12))
        if root + 1 != nl:
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "root level does not match level count")
        return cls(levels, sg, res, root, st, child_type), offset

    # ---- .svo (export_import_structure.cpp:15-45)
    def to_svo_bytes(self) -> bytes:
        assert self.child_type == "u32"
        return struct.pack("<II", SVO_MAGIC, SVO_VERSION) + self.to_bytes()

    @classmethod
    def from_svo_bytes(cls, buf: bytes) -> "EditStructure":
        if len(buf) < 8:
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "truncated .svo")
        magic, version = struct.unpack("<II", buf[:8])
        if magic != SVO_MAGIC or version != SVO_VERSION:
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "bad .svo magic/version")
        s, off = cls.from_bytes(buf, 8)
        if off != len(buf):
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "trailing bytes in .svo")
        return s

    def compute_voxel_count(self) -> int:
        """computeVoxelCount (structure.h:453-481): voxels of the expanded tree."""
        if self.root_level < 3 or len(self.nodes_per_level[self.root_level]) == 0:
            return 0
        leaf_pc = np.array([bin(int(v)).count("1") for v in self.sub_grids], dtype=np.int64) if len(self.sub_grids) else np.zeros(0, np.int64)
        counts = leaf_pc
        for lvl in range(3, self.root_level + 1):
            nodes = self.nodes_per_level[lvl].astype(np.int64)
            empty = nodes == EMPTY_CHILD
            safe = np.where(empty, 0, nodes)
            counts = np.where(empty, 0, counts[safe] if len(counts) else 0).sum(axis=1)
        return int(counts[0])


def write_tdag(structure: EditStructure, config: TransformDAGConfig) -> bytes:
    """.tdag: EditStructure<void, TransformPointer> then the raw TransformDAGConfig
    (voxelizer/src/main.cpp:144-151)."""
    assert structure.child_type == "transform"
    return structure.to_bytes() + config.to_bytes()


def read_tdag(buf: bytes):
    s, off = EditStructure.from_bytes(buf, 0, child_type="transform")
    cfg = TransformDAGConfig.from_bytes(buf[off: off + 8]) if len(buf) >= off + 8 else None
    return s, cfg


# ------------------------------------------------------------------------------------------------
# Context + construction entry points
# ------------------------------------------------------------------------------------------------
class Context:
    """One CUDA device + stream (tdag_ctx)."""

    def __init__(self, device: int = 0, tuning: Optional[dict] = None):
        L = lib()
        t = _abi.Tuning()
        for k, v in (tuning or {}).items():
            setattr(t, k, v)
        self._ptr = ctypes.c_void_p()
        _abi.check(L.tdag_ctx_create(device, ctypes.byref(t), ctypes.byref(self._ptr)))
        self.device = device

    @property
    def handle(self):
        return self._ptr

    def close(self):
        if self._ptr:
            lib().tdag_ctx_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("TDAG_DEVICE", "0")))
    return _default_ctx


def _config_struct(cfg: TransformDAGConfig) -> _abi.Config:
    c = _abi.Config()
    c.symmetry = int(cfg.symmetry)
    c.axis_permutation = int(cfg.axis_permutation)
    c.translation = int(cfg.translation)
    c.max_translation_level = int(cfg.max_translation_level)
    return c


def _view_of(dag: EditStructure, keep: list) -> _abi.SvdagView:
    v = _abi.SvdagView()
    v.resolution = dag.resolution
    v.root_level = dag.root_level
    v.structure_type = dag.structure_type
    for lvl in range(3, dag.root_level + 1):
        a = np.ascontiguousarray(dag.nodes_per_level[lvl], dtype=np.uint32)
        keep.append(a)
        v.nodes[lvl] = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        v.node_counts[lvl] = a.shape[0]
    sg = np.ascontiguousarray(dag.sub_grids, dtype=np.uint64)
    keep.append(sg)
    v.leaves = sg.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    v.leaf_count = sg.shape[0]
    return v


def _take_result(rp) -> (EditStructure, dict):
    r = rp.contents
    try:
        levels = []
        for lvl in range(r.root_level + 1):
            cnt = r.node_counts[lvl]
            if lvl >= 3 and cnt:
                a = np.ctypeslib.as_array(r.nodes[lvl], shape=(cnt * 8,)).copy().reshape(cnt, 8)
            else:
                a = np.zeros((0, 8), dtype=np.uint64)
            levels.append(a)
        leaves = np.ctypeslib.as_array(r.leaves, shape=(r.leaf_count,)).copy() if r.leaf_count else np.zeros(0, np.uint64)
        stats = _abi.stats_to_dict(r.stats, r.root_level)
        return EditStructure(levels, leaves, r.resolution, r.root_level, r.structure_type, "transform"), stats
    finally:
        lib().tdag_result_free(rp)


def construct_transform_dag(in_dag: EditStructure, config: TransformDAGConfig = TransformDAGConfig(),
                            ctx: Optional[Context] = None, return_stats: bool = False):
    """constructTransformDAG (transform_dag.h:161-162): returns EditStructure<void, TransformPointer>.
    Raises TDagError like the reference's assert_always when the input is not a DAG."""
    ctx = ctx or default_context()
    keep = []
    view = _view_of(in_dag, keep)
    rp = ctypes.POINTER(_abi.Result)()
    _abi.check(lib().tdag_build(ctx.handle, ctypes.byref(view), ctypes.byref(_config_struct(config)), ctypes.byref(rp)))
    out, stats = _take_result(rp)
    return (out, stats) if return_stats else out


def construct_transform_dag_hierarchical(in_dag: EditStructure, config: TransformDAGConfig = TransformDAGConfig(),
                                         ctx: Optional[Context] = None) -> EditStructure:
    """constructTransformDAGHierarchical(inDag, config) (transform_dag.h:168-169)."""
    ctx = ctx or default_context()
    keep = []
    view = _view_of(in_dag, keep)
    rp = ctypes.POINTER(_abi.Result)()
    _abi.check(lib().tdag_build_hierarchical(ctx.handle, ctypes.byref(view), ctypes.byref(_config_struct(config)), ctypes.byref(rp)))
    return _take_result(rp)[0]


def find_duplicates_among_flattened_items(level: int, grids: np.ndarray, config: TransformDAGConfig = TransformDAGConfig(),
                                          ctx: Optional[Context] = None, return_stats: bool = False):
    """findDuplicatesAmongFlattenedItems_cpp2<level> (transform_dag.h:307-308) on dense grids
    (n x R^3/64 uint64, bit x + R*y + R*R*z). Returns (unique positions, mapping TransformPointers)."""
    ctx = ctx or default_context()
    g = np.ascontiguousarray(grids, dtype=np.uint64)
    n = g.shape[0]
    mapping = np.zeros(n, np.uint64)
    uniq = np.zeros(max(n, 1), np.uint32)
    nu = ctypes.c_uint32()
    st = _abi.LevelStats()
    _abi.check(lib().tdag_find_duplicates_level(ctx.handle, level, g.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n,
                                                ctypes.byref(_config_struct(config)),
                                                mapping.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                                uniq.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(nu),
                                                ctypes.byref(st)))
    res = (uniq[: nu.value].copy(), mapping)
    return (res + (_abi.level_stats_to_dict(st),)) if return_stats else res


# ------------------------------------------------------------------------------------------------
# Device-side input pipeline: scenes, SVO build, toDAG (device-resident EditStructure<void, uint32_t>)
# ------------------------------------------------------------------------------------------------
SCENE_TERRAIN = 0
SCENE_PRIMITIVES = 1


@dataclasses.dataclass
class SceneSpec:
    """tdag_scene: a procedural grid generated on the device."""

    kind: int = SCENE_PRIMITIVES
    resolution: int = 2048
    seed: int = 1
    num_primitives: int = 4000
    copy_percent: int = 30
    shell: bool = True
    chunk_resolution: int = 0  # 0: automatic (chunked above 4096^3); else generated in chunks of this size

    def to_c(self) -> _abi.Scene:
        c = _abi.Scene()
        c.kind, c.resolution, c.seed = self.kind, self.resolution, self.seed
        c.num_primitives, c.copy_percent, c.shell = self.num_primitives, self.copy_percent, int(self.shell)
        c.chunk_resolution = self.chunk_resolution
        return c


def scene_primitives(spec: SceneSpec) -> list:
    """The deterministic primitive list of a scene (tdag_scene_primitives)."""
    c = spec.to_c()
    n = ctypes.c_uint32()
    _abi.check(lib().tdag_scene_primitives(ctypes.byref(c), None, 0, ctypes.byref(n)))
    arr = (_abi.Primitive * max(1, n.value))()
    _abi.check(lib().tdag_scene_primitives(ctypes.byref(c), arr, n.value, ctypes.byref(n)))
    out = []
    for i in range(n.value):
        p = arr[i]
        out.append({"type": p.type, "xform": p.xform, "size": tuple(p.size), "radius": p.radius,
                    "offset": tuple(p.offset), "seed": p.seed, "source": p.source})
    return out


class DeviceSvdag:
    """A library-owned device-resident EditStructure<void, uint32_t> (tdag_svdag)."""

    def __init__(self, handle: ctypes.c_void_p, ctx: Context):
        self._h = handle
        self._ctx = ctx

    @property
    def handle(self):
        return self._h

    def view(self) -> _abi.SvdagView:
        v = _abi.SvdagView()
        _abi.check(lib().tdag_svdag_get_view(self._h, ctypes.byref(v)))
        return v

    @property
    def voxel_count(self) -> int:
        n = ctypes.c_uint64()
        _abi.check(lib().tdag_svdag_voxel_count(self._h, ctypes.byref(n)))
        return n.value

    def to_host(self) -> EditStructure:
        v = self.view()
        levels = []
        for lvl in range(v.root_level + 1):
            cnt = v.node_counts[lvl] if lvl >= 3 else 0
            a = np.zeros((cnt, 8), np.uint32)
            if cnt:
                _abi.check(lib().tdag_svdag_copy_level(self._ctx.handle, self._h, lvl, a.ctypes.data, a.nbytes))
            levels.append(a)
        leaves = np.zeros(v.leaf_count, np.uint64)
        if v.leaf_count:
            _abi.check(lib().tdag_svdag_copy_level(self._ctx.handle, self._h, 2, leaves.ctypes.data, leaves.nbytes))
        return EditStructure(levels, leaves, v.resolution, v.root_level, v.structure_type, "u32")

    def free(self):
        if self._h:
            lib().tdag_svdag_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def scene_svdag(spec: SceneSpec, to_dag: bool = True, ctx: Optional[Context] = None) -> DeviceSvdag:
    ctx = ctx or default_context()
    h = ctypes.c_void_p()
    c = spec.to_c()
    _abi.check(lib().tdag_scene_svdag(ctx.handle, ctypes.byref(c), int(to_dag), ctypes.byref(h)))
    return DeviceSvdag(h, ctx)


def scene_svdag_checkpointed(spec: SceneSpec, path: str, every_chunks: int = 0, stop_after_chunks: int = 0,
                             ctx: Optional[Context] = None) -> DeviceSvdag:
    """scene_svdag of a streamed scene with checkpoints (tdag_scene_svdag_checkpointed): resumes from
    `path` when it holds a checkpoint of the same scene, writes one every `every_chunks` chunks, and
    with stop_after_chunks raises TDagError (TDAG_ERR_INTERRUPTED) after that many chunks, checkpoint
    written."""
    ctx = ctx or default_context()
    h = ctypes.c_void_p()
    c = spec.to_c()
    _abi.check(lib().tdag_scene_svdag_checkpointed(ctx.handle, ctypes.byref(c), os.fsencode(path), every_chunks, stop_after_chunks,
                                                   ctypes.byref(h)))
    return DeviceSvdag(h, ctx)


def svdag_from_dense(dense: np.ndarray, to_dag: bool = True, ctx: Optional[Context] = None) -> DeviceSvdag:
    """EditStructure(VoxelGrid) (+ toDAG) on the device; dense[z, y, x] (x fastest)."""
    ctx = ctx or default_context()
    d = np.ascontiguousarray(dense, dtype=np.uint8)
    h = ctypes.c_void_p()
    _abi.check(lib().tdag_svdag_from_dense(ctx.handle, d.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), d.shape[0],
                                           int(to_dag), ctypes.byref(h)))
    return DeviceSvdag(h, ctx)


class DeviceResult:
    """A device-resident EditStructure<void, TransformPointer> (tdag_result with on_device = 1)."""

    def __init__(self, rp):
        self._rp = rp
        self.stats = _abi.stats_to_dict(rp.contents.stats, rp.contents.root_level)

    def to_host(self, ctx: Optional[Context] = None) -> EditStructure:
        """Host copy of the device-resident result (tdag_result_to_host)."""
        ctx = ctx or default_context()
        hp = ctypes.POINTER(_abi.Result)()
        _abi.check(lib().tdag_result_to_host(ctx.handle, self._rp, ctypes.byref(hp)))
        return _take_result(hp)[0]

    def free(self):
        if self._rp:
            lib().tdag_result_free(self._rp)
            self._rp = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def construct_transform_dag_device(in_dag: DeviceSvdag, config: TransformDAGConfig = TransformDAGConfig(),
                                   ctx: Optional[Context] = None) -> DeviceResult:
    """constructTransformDAG with the input and the result resident in device memory (tdag_build_device)."""
    ctx = ctx or default_context()
    v = in_dag.view()
    rp = ctypes.POINTER(_abi.Result)()
    _abi.check(lib().tdag_build_device(ctx.handle, ctypes.byref(v), ctypes.byref(_config_struct(config)), ctypes.byref(rp)))
    return DeviceResult(rp)


def construct_transform_dag_batched(dags: List[EditStructure], config: TransformDAGConfig = TransformDAGConfig(),
                                    ctx: Optional[Context] = None, return_stats: bool = False):
    """Batched constructTransformDAG (tdag_build_batched): one pass over all structures, result i equal
    to construct_transform_dag(dags[i]) bit for bit."""
    ctx = ctx or default_context()
    keep = []
    views = (_abi.SvdagView * max(1, len(dags)))()
    for i, d in enumerate(dags):
        views[i] = _view_of(d, keep)
    outs = (ctypes.POINTER(_abi.Result) * max(1, len(dags)))()
    st = _abi.Stats()
    _abi.check(lib().tdag_build_batched(ctx.handle, views, len(dags), ctypes.byref(_config_struct(config)), outs, ctypes.byref(st)))
    results = [_take_result(outs[i])[0] for i in range(len(dags))]
    if return_stats:
        return results, _abi.stats_to_dict(st, max((d.root_level for d in dags), default=2))
    return results


def construct_transform_dag_batched_device(dags: List["DeviceSvdag"], config: TransformDAGConfig = TransformDAGConfig(),
                                           ctx: Optional[Context] = None):
    """tdag_build_batched_device: device-resident inputs and results. Returns (results, batch stats)."""
    ctx = ctx or default_context()
    views = (_abi.SvdagView * max(1, len(dags)))()
    root = 2
    for i, d in enumerate(dags):
        views[i] = d.view()
        root = max(root, views[i].root_level)
    outs = (ctypes.POINTER(_abi.Result) * max(1, len(dags)))()
    st = _abi.Stats()
    _abi.check(lib().tdag_build_batched_device(ctx.handle, views, len(dags), ctypes.byref(_config_struct(config)), outs, ctypes.byref(st)))
    return [DeviceResult(outs[i]) for i in range(len(dags))], _abi.stats_to_dict(st, root)


class BatchGraph:
    """A batched build captured in one CUDA graph (tdag_batch_graph_create / _launch / _free).

    Creation builds the device-resident batch once, recording every value the build reads back, and
    captures the same build into a graph; ``launch()`` replays it in one cudaGraphLaunch and returns
    the device results (equal to construct_transform_dag_batched_device's) and the stats. The batch's
    arrays must keep their contents: a launch on changed arrays raises TDagError (TDAG_ERR_ARG)."""

    def __init__(self, dags: List["DeviceSvdag"], config: TransformDAGConfig = TransformDAGConfig(), ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.dags = list(dags)  # the inputs stay alive with the graph
        self.count = len(self.dags)
        views = (_abi.SvdagView * max(1, self.count))()
        self.root = 2
        for i, d in enumerate(self.dags):
            views[i] = d.view()
            self.root = max(self.root, views[i].root_level)
        h = ctypes.c_void_p()
        _abi.check(lib().tdag_batch_graph_create(self.ctx.handle, views, self.count, ctypes.byref(_config_struct(config)), ctypes.byref(h)))
        self.handle = h

    def launch(self):
        outs = (ctypes.POINTER(_abi.Result) * max(1, self.count))()
        st = _abi.Stats()
        _abi.check(lib().tdag_batch_graph_launch(self.handle, outs, ctypes.byref(st)))
        return [DeviceResult(outs[i]) for i in range(self.count)], _abi.stats_to_dict(st, self.root)

    def free(self):
        if getattr(self, "handle", None):
            lib().tdag_batch_graph_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------------
# .tdag16 encoding (include/tdag16.h)
# ------------------------------------------------------------------------------------------------
def _host_result_view(dag: EditStructure, keep: list) -> _abi.Result:
    r = _abi.Result()
    r.resolution = dag.resolution
    r.root_level = dag.root_level
    r.structure_type = dag.structure_type
    r.on_device = 0
    for lvl in range(3, dag.root_level + 1):
        a = np.ascontiguousarray(dag.nodes_per_level[lvl], dtype=np.uint64)
        keep.append(a)
        r.nodes[lvl] = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        r.node_counts[lvl] = a.shape[0]
    sg = np.ascontiguousarray(dag.sub_grids, dtype=np.uint64)
    keep.append(sg)
    r.leaves = sg.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    r.leaf_count = sg.shape[0]
    return r


def construct_transform_dag16(dag, dag_config: TransformDAGConfig = TransformDAGConfig(),
                              encoding_config: TransformEncodingConfig = TransformEncodingConfig(),
                              ctx: Optional[Context] = None, return_stats: bool = False):
    """constructTransformDAG16(EditStructure<void, TransformPointer>, dagConfig, encodingConfig, stats)
    (tools/svdag_encoding/src/transform_dag_encoding.cpp:240-497) followed by TransformDAG16::writeTo:
    returns the .tdag16 file bytes (and, with return_stats, the per-level DAGEncodingStats).
    ``dag`` is a host EditStructure of TransformPointers, a DeviceResult, or a StaticStructure of
    TransformPointers (constructTransformDAG16(StaticStructure<void, TransformPointer>, ...),
    transform_dag_encoding.cpp:519-697, which makes the same decisions on the unpacked structure; only
    its statistics are indexed by child level there)."""
    ctx = ctx or default_context()
    keep = []
    if isinstance(dag, StaticStructure):
        dag = dag.to_edit()
    if isinstance(dag, DeviceResult):
        rp_in = dag._rp
    else:
        rp_in = ctypes.pointer(_host_result_view(dag, keep))
    enc = _abi.EncodingConfig(int(encoding_config.pointer_tables), int(encoding_config.huffman_code), encoding_config.tie_code())
    op = ctypes.POINTER(_abi.Tdag16Result)()
    _abi.check(lib().tdag_encode16(ctx.handle, rp_in, ctypes.byref(_config_struct(dag_config)), ctypes.byref(enc), ctypes.byref(op)))
    try:
        r = op.contents
        data = ctypes.string_at(r.bytes, r.size)
        stats = {
            "encode_ms": r.encode_ms, "wall_ms": r.wall_ms, "kernel_launches": r.kernel_launches,
            "levels": {l: {k: (list(getattr(r.levels[l], k)) if k in ("table_pointers", "direct_pointers") else getattr(r.levels[l], k))
                           for k, _ in _abi.Tdag16LevelStats._fields_} for l in range(2, r.root_level + 1)},
        }
    finally:
        lib().tdag16_result_free(op)
    return (data, stats) if return_stats else data


def encoding_stats_json(stats: dict, total_size_in_bytes: int, dag_config: TransformDAGConfig = TransformDAGConfig(),
                        encoding_config: TransformEncodingConfig = TransformEncodingConfig()) -> dict:
    """The svdag_encoding tool's --stats JSON (DAGEncodingStats::write and LevelStats' conversion,
    tools/svdag_encoding/src/transform_dag_encoding.cpp:58-82) from construct_transform_dag16's
    stats: one entry per tree level 0 .. root (zeros below the leaves), the file size and both configs."""
    root = max(stats["levels"]) if stats["levels"] else 0
    pt = bool(encoding_config.pointer_tables)
    levels = []
    for l in range(root + 1):
        st = stats["levels"].get(l)
        if st is None:
            levels.append({"num_table_pointers_of_size_u16": [0, 0, 0], "num_direct_pointers_of_size_u16": [0, 0, 0],
                           "table_size_in_pointers": 0, "pointer_size_in_table": 0, "num_nodes": 0, "memory_in_bytes": 0})
            continue
        node_level = l >= 3  # the pointer statistics belong to the node level whose children they point to
        levels.append({"num_table_pointers_of_size_u16": [int(v) for v in st["table_pointers"]],
                       "num_direct_pointers_of_size_u16": [int(v) for v in st["direct_pointers"]],
                       "table_size_in_pointers": int(st["table_size"]) if (pt and node_level) else 0,
                       "pointer_size_in_table": 8 if (pt and node_level) else 0,
                       "num_nodes": int(st["num_nodes"]), "memory_in_bytes": int(st["memory_in_bytes"])})
    return {"levels": levels, "total_size_in_bytes": int(total_size_in_bytes), "pointer_tables": pt,
            "huffman_code": bool(encoding_config.huffman_code), "symmetry": bool(dag_config.symmetry),
            "axis_permutation": bool(dag_config.axis_permutation), "enable_translation": bool(dag_config.translation),
            "translation_level": int(dag_config.max_translation_level)}


def create_length_limited_huffman_code_table(frequencies, max_code_length: int = 16, lsb_first: bool = False):
    """createLengthLimitedHuffmanCodeTable (+ convertHuffmanToLSB when lsb_first) (huffman.cpp:165-182):
    a list of (code, bits) per symbol. Host computation in libtdag.so."""
    f = np.ascontiguousarray(frequencies, dtype=np.uint64)
    codes = np.zeros(len(f), np.uint64)
    bits = np.zeros(len(f), np.uint32)
    _abi.check(lib().tdag16_huffman_code_table(f.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(f), int(max_code_length),
                                               int(lsb_first), codes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                               bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
    return [(int(c), int(b)) for c, b in zip(codes, bits)]


class Tdag16Device:
    """A .tdag16 file resident in device memory (tdag16_upload), for voxel queries
    (TransformDAG16::get) and the lossless check against its source SVDAG."""

    def __init__(self, data: bytes, ctx: Optional[Context] = None):
        self._ctx = ctx or default_context()
        buf = np.frombuffer(data, dtype=np.uint8)
        h = ctypes.c_void_p()
        _abi.check(lib().tdag16_upload(self._ctx.handle, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(data), ctypes.byref(h)))
        self._h = h

    def get(self, xyz):
        """Occupancy of n voxels: xyz is an (n, 3) integer array (host) or a CUDA uint32/int32 tensor."""
        import torch
        on_host = not (isinstance(xyz, torch.Tensor) and xyz.is_cuda)
        t = torch.as_tensor(np.ascontiguousarray(xyz, dtype=np.uint32).view(np.int32)) if on_host else xyz
        t = t.to(device="cuda", dtype=torch.int32).contiguous()
        n = t.shape[0]
        out = torch.empty(n, dtype=torch.uint8, device=t.device)
        torch.cuda.synchronize()
        _abi.check(lib().tdag16_get(self._ctx.handle, self._h, ctypes.c_void_p(t.data_ptr()), n, ctypes.c_void_p(out.data_ptr())))
        return out.cpu().numpy() if on_host else out

    def raycast(self, rays):
        """First solid voxel per ray: rays is an (n, 8) float32 array (origin xyz, direction xyz, tmin,
        tmax) on the host or a CUDA tensor. Returns (t, voxel (n, 3), hit, steps) as numpy arrays."""
        import torch
        r = rays if (isinstance(rays, torch.Tensor) and rays.is_cuda) else torch.as_tensor(np.ascontiguousarray(rays, dtype=np.float32))
        r = r.to(device="cuda", dtype=torch.float32).contiguous()
        n = r.shape[0]
        out = torch.empty((n, 6), dtype=torch.int32, device=r.device)  # tdag16_hit: t, voxel[3], hit, steps
        torch.cuda.synchronize()
        _abi.check(lib().tdag16_raycast(self._ctx.handle, self._h, ctypes.c_void_p(r.data_ptr()), n, ctypes.c_void_p(out.data_ptr())))
        o = out.cpu().numpy()
        return o[:, 0].copy().view(np.float32), o[:, 1:4].astype(np.uint32), o[:, 4].astype(np.uint8), o[:, 5].astype(np.uint32)

    def verify(self, source: "DeviceSvdag") -> dict:
        """Lossless check against the device SVDAG the DAG was built from (tdag16_verify)."""
        st = _abi.Tdag16VerifyStats()
        v = source.view()
        _abi.check(lib().tdag16_verify(self._ctx.handle, self._h, ctypes.byref(v), ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _abi.Tdag16VerifyStats._fields_ if k != "reserved"}

    def free(self):
        if getattr(self, "_h", None):
            lib().tdag16_device_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------------
# StaticStructure (structure.h:298-320, 765-798, 859-895) and constructStaticTransformDAG
# ------------------------------------------------------------------------------------------------
@dataclasses.dataclass
class StaticStructure:
    """StaticStructure<void, Child>: ``words[l]`` is level l's packed word stream (uint32 for
    ``child_type="u32"``, uint64 TransformPointers for ``"transform"``): per node a header word (child
    mask) and one word per present child, the child's word offset in level l-1 (leaf index at level 3)."""

    words: List[np.ndarray]
    sub_grids: np.ndarray
    resolution: int
    root_level: int
    structure_type: int = 0
    child_type: str = "u32"

    @property
    def word_dtype(self):
        return np.uint32 if self.child_type == "u32" else np.uint64

    @classmethod
    def from_edit(cls, e: EditStructure) -> "StaticStructure":
        """StaticStructure(const EditStructure&) (structure.h:765-798)."""
        is_tp = e.child_type == "transform"
        dt = np.uint64 if is_tp else np.uint32
        empty = np.uint64(tp_create(0xFFFFFFFF)) if is_tp else np.uint32(0xFFFFFFFF)
        ptr_mask = np.uint64((1 << 37) - 1)
        prev = np.arange(len(e.sub_grids), dtype=np.uint64)
        words = [np.zeros(0, dt) for _ in range(len(e.nodes_per_level))]
        for lvl in range(3, e.root_level + 1):
            nodes = np.asarray(e.nodes_per_level[lvl], dtype=dt).reshape(-1, 8)
            present = nodes != empty
            sizes = 1 + present.sum(axis=1)
            starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
            w = np.zeros(int(sizes.sum()), dt)
            w[starts.astype(np.int64)] = (present.astype(dt) << np.arange(8, dtype=dt)).sum(axis=1).astype(dt)
            rank = np.cumsum(present, axis=1) - 1
            r, k = np.nonzero(present)
            pos = (starts[r] + 1 + rank[r, k].astype(np.uint64)).astype(np.int64)
            c = nodes[r, k]
            if is_tp:
                w[pos] = (c & ~ptr_mask) | prev[(c & ptr_mask).astype(np.int64)]
            else:
                w[pos] = prev[c.astype(np.int64)].astype(dt)
            words[lvl] = w
            prev = starts
        return cls(words, np.asarray(e.sub_grids, np.uint64).copy(), e.resolution, e.root_level, e.structure_type, e.child_type)

    def to_edit(self) -> EditStructure:
        """The same structure with fixed 8-child nodes: node starts by a sequential walk of each level
        (getLevelNodeStarts, structure.h:859-876), child word offsets turned into node indices."""
        is_tp = self.child_type == "transform"
        dt = np.uint64 if is_tp else np.uint32
        empty = tp_create(0xFFFFFFFF) if is_tp else 0xFFFFFFFF
        ptr_mask = (1 << 37) - 1
        levels = [np.zeros((0, 8), dt) for _ in range(len(self.words))]
        prev_index = None  # word offset -> node index of the level below (level 3: leaf indices)
        for lvl in range(3, self.root_level + 1):
            w = [int(v) for v in np.asarray(self.words[lvl])]
            nodes, index, at = [], {}, 0
            while at < len(w):
                mask = w[at] & 0xFF
                index[at] = len(nodes)
                row, c = [empty] * 8, at + 1
                for k in range(8):
                    if (mask >> k) & 1:
                        if c >= len(w):
                            raise TDagError(_abi.TDAG_ERR_CORRUPT, "static node runs past its level")
                        v = w[c]
                        off = (v & ptr_mask) if is_tp else v
                        idx = off if lvl == 3 else prev_index.get(off)
                        if idx is None:
                            raise TDagError(_abi.TDAG_ERR_CORRUPT, "static child pointer is not a node start")
                        row[k] = ((v & ~ptr_mask) | idx) if is_tp else idx
                        c += 1
                nodes.append(row)
                at = c
            levels[lvl] = np.array(nodes, dtype=dt).reshape(-1, 8)
            prev_index = index
        return EditStructure(levels, np.asarray(self.sub_grids, np.uint64).copy(), self.resolution, self.root_level,
                             self.structure_type, self.child_type)

    def to_bytes(self) -> bytes:
        """StaticStructure::writeTo (structure.h:887-895)."""
        out = [struct.pack("<Q", len(self.words))]
        for w in self.words:
            a = np.ascontiguousarray(w, dtype=self.word_dtype)
            out.append(struct.pack("<Q", a.shape[0]))
            out.append(a.tobytes())
        sg = np.ascontiguousarray(self.sub_grids, dtype=np.uint64)
        out.append(struct.pack("<Q", sg.shape[0]))
        out.append(sg.tobytes())
        out.append(struct.pack("<III", self.resolution, self.root_level, self.structure_type))
        return b"".join(out)

    @classmethod
    def from_bytes(cls, buf: bytes, child_type: str = "u32") -> "StaticStructure":
        dt = np.uint32 if child_type == "u32" else np.uint64
        off = 0

        def take(n):
            nonlocal off
            if off + n > len(buf):
                raise TDagError(_abi.TDAG_ERR_CORRUPT, "truncated static structure")
            b = buf[off: off + n]
            off += n
            return b

        (nl,) = struct.unpack("<Q", take(8))
        if nl > 64:
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "corrupt level count")
        words = []
        for _ in range(nl):
            (cnt,) = struct.unpack("<Q", take(8))
            words.append(np.frombuffer(take(cnt * np.dtype(dt).itemsize), dtype=dt).copy())
        (cnt,) = struct.unpack("<Q", take(8))
        sg = np.frombuffer(take(cnt * 8), dtype=np.uint64).copy()
        res, root, st = struct.unpack("<III", take(12))
        if root + 1 != nl or off != len(buf):
            raise TDagError(_abi.TDAG_ERR_CORRUPT, "malformed static structure")
        return cls(words, sg, res, root, st, child_type)


def construct_static_transform_dag(in_dag: StaticStructure, config: TransformDAGConfig = TransformDAGConfig(),
                                   ctx: Optional[Context] = None, return_stats: bool = False):
    """constructStaticTransformDAG (transform_dag.h:163; transform_dag.cpp:242-390): returns a
    StaticStructure of TransformPointers."""
    assert in_dag.child_type == "u32"
    ctx = ctx or default_context()
    v = _abi.StaticView()
    v.resolution, v.root_level, v.structure_type = in_dag.resolution, in_dag.root_level, in_dag.structure_type
    keep = []
    for lvl in range(3, in_dag.root_level + 1):
        a = np.ascontiguousarray(in_dag.words[lvl], dtype=np.uint32)
        keep.append(a)
        v.words[lvl] = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        v.word_counts[lvl] = a.shape[0]
    sg = np.ascontiguousarray(in_dag.sub_grids, dtype=np.uint64)
    keep.append(sg)
    v.leaves = sg.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    v.leaf_count = sg.shape[0]
    rp = ctypes.POINTER(_abi.StaticResult)()
    _abi.check(lib().tdag_build_static(ctx.handle, ctypes.byref(v), ctypes.byref(_config_struct(config)), ctypes.byref(rp)))
    try:
        r = rp.contents
        words = []
        for lvl in range(r.root_level + 1):
            cnt = r.word_counts[lvl]
            words.append(np.ctypeslib.as_array(r.words[lvl], shape=(cnt,)).copy() if (lvl >= 3 and cnt) else np.zeros(0, np.uint64))
        leaves = np.ctypeslib.as_array(r.leaves, shape=(r.leaf_count,)).copy() if r.leaf_count else np.zeros(0, np.uint64)
        out = StaticStructure(words, leaves, r.resolution, r.root_level, r.structure_type, "transform")
        stats = _abi.stats_to_dict(r.stats, r.root_level)
    finally:
        lib().tdag_static_result_free(rp)
    return (out, stats) if return_stats else out
