"""Test helpers: seeded inputs built with the oracle's SVO builder and toDAG."""
import numpy as np


def random_grid(res, density, seed):
    rng = np.random.default_rng(seed)
    return (rng.random((res, res, res)) < density).astype(np.uint8)


def blocky_grid(res, seed, n_boxes=12, max_side=None):
    """Union of random boxes plus mirrored/translated copies: many exact matches."""
    rng = np.random.default_rng(seed)
    g = np.zeros((res, res, res), np.uint8)
    max_side = max_side or max(2, res // 3)
    for _ in range(n_boxes):
        s = rng.integers(1, max_side + 1, size=3)
        o = [rng.integers(0, res - s[k] + 1) for k in range(3)]
        g[o[2]:o[2] + s[2], o[1]:o[1] + s[1], o[0]:o[0] + s[0]] = 1
    # copy an octant with a mirror and a shift, to create transform matches
    h = res // 2
    block = g[:h, :h, :h].copy()
    g[h:, h:, :h] |= block[:, ::-1, :]
    g[:h, h:, h:] |= np.transpose(block, (1, 0, 2))
    return g


def dag_svo_bytes(oracle, dense):
    return oracle.to_dag(oracle.svo_from_dense(dense))


def structure_from_svo(tdag_mod, svo_bytes):
    return tdag_mod.EditStructure.from_svo_bytes(svo_bytes)


def synthetic_tdag(n_leaves, refs_per_leaf, seed):
    """A transform DAG whose level-3 nodes reference n_leaves distinct (leaf, transform) pointers
    refs_per_leaf times each, in a random order, under an 8-ary tree up to a single root."""
    import tdag
    rng = np.random.default_rng(seed)
    leaves = rng.integers(1, 2**63, size=n_leaves, dtype=np.uint64)
    ptrs = []
    for i in range(n_leaves):
        t = rng.integers(-3, 4, size=3) * (rng.random() < 0.5)
        ptrs.append(tdag.tp_create(i, tuple(bool(b) for b in rng.integers(0, 2, 3)), [(0, 1, 2), (1, 2, 0), (2, 1, 0)][i % 3],
                                   tuple(int(v) for v in t)))
    refs = np.repeat(np.array(ptrs, dtype=np.uint64), refs_per_leaf)
    rng.shuffle(refs)
    levels = [np.zeros((0, 8), np.uint64)] * 3
    sentinel = tdag.tp_create(0xFFFFFFFF)
    n3 = -(-len(refs) // 8)
    l3 = np.full(n3 * 8, sentinel, dtype=np.uint64)
    l3[: len(refs)] = refs
    levels.append(l3.reshape(n3, 8))
    count = n3
    while count > 1:
        up = -(-count // 8)
        lv = np.full(up * 8, sentinel, dtype=np.uint64)
        lv[:count] = [tdag.tp_create(i) for i in range(count)]
        levels.append(lv.reshape(up, 8))
        count = up
    root = len(levels) - 1
    s = tdag.EditStructure(levels, leaves, 1 << root, root, 0, "transform")
    return tdag.write_tdag(s, tdag.TransformDAGConfig()), s


def mask_tdag16_padding(data: bytes) -> bytes:
    """A .tdag16 with the bytes that the reference leaves uninitialised set to zero.

    TransformDAG16::writeTo (transform_dag_encoding.cpp:1023-1030) writes two structs raw:
    TransformDAGConfig (three bools, one padding byte, a uint32_t; transform_dag.h:157-160) and,
    in each Huffman decoder, the vector of ``Code {uint64_t code; uint32_t bits;}`` (huffman.h:12-17),
    whose last 4 of 16 bytes are padding. Only those bytes are cleared."""
    b = bytearray(data)
    b[3] = 0
    off = 8 + 2  # TransformDAGConfig, TransformEncodingConfig
    rd = lambda o, n: int.from_bytes(b[o:o + n], "little")
    levels = rd(off, 8)
    off += 8
    for _ in range(levels):
        off += 8 + 2 * rd(off, 8)
    off += 8 + 8 * rd(off, 8)  # leaves
    off += 4 + 4  # resolution, rootLevel
    tables = rd(off, 8)
    off += 8
    for _ in range(tables):
        off += 8 + 8 * rd(off, 8)
    luts = rd(off, 8)
    off += 8
    for _ in range(luts):
        n = rd(off, 8)
        off += 8
        for i in range(n):
            b[off + 16 * i + 12: off + 16 * i + 16] = b"\0\0\0\0"
        off += 16 * n
    if off != len(b):
        raise ValueError(f".tdag16 layout: parsed {off} of {len(b)} bytes")
    return bytes(b)
