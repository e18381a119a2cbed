"""CPU tests of the oracle: the reference's own structure test cases, restated, and
self-consistency properties of the Transform-DAG restatement."""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid


def morton3(x, y, z):
    def part(v):
        r = 0
        for b in range(10):
            r |= ((v >> b) & 1) << (3 * b)
        return r
    return part(x) | (part(y) << 1) | (part(z) << 2)


def svo_get(structure, x, y, z):
    """EditStructure::get (structure.h:600-625): Morton child index per level, leaf bit Morton(v & 3)."""
    node = 0
    for level in range(structure.root_level, 2, -1):
        child_level = level - 1
        c = morton3((x >> child_level) & 1, (y >> child_level) & 1, (z >> child_level) & 1)
        node = int(structure.nodes_per_level[level][node][c])
        if node == 0xFFFFFFFF:
            return False
    bit = morton3(x & 3, y & 3, z & 3)
    return bool((int(structure.sub_grids[node]) >> bit) & 1)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_structure_from_voxel_grid_random16(oracle, seed):
    """tools/lib/tests/src/voxel/structure.cpp:69-92: random 16^3 grid -> EditStructure(VoxelGrid) -> get()."""
    import tdag
    rng = np.random.default_rng(seed)
    dense = rng.integers(0, 2, size=(16, 16, 16), dtype=np.uint8)
    s = tdag.EditStructure.from_svo_bytes(oracle.svo_from_dense(dense))
    assert s.resolution == 16 and s.root_level == 4 and len(s.nodes_per_level) == 5
    assert all(len(s.nodes_per_level[l]) == 0 for l in range(3))
    for z in range(16):
        for y in range(16):
            for x in range(16):
                assert svo_get(s, x, y, z) == bool(dense[z, y, x])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_svo_save_load_roundtrip(oracle, seed):
    """tools/lib/tests/src/voxel/save_structure.cpp:9-36: export -> import equals the original."""
    import tdag
    dense = np.random.default_rng(100 + seed).integers(0, 2, size=(16, 16, 16), dtype=np.uint8)
    svo = oracle.svo_from_dense(dense)
    s = tdag.EditStructure.from_svo_bytes(svo)
    assert s.to_svo_bytes() == svo
    s2 = tdag.EditStructure.from_svo_bytes(s.to_svo_bytes())
    assert s2.resolution == s.resolution and s2.structure_type == s.structure_type
    for a, b in zip(s.nodes_per_level, s2.nodes_per_level):
        assert np.array_equal(a, b)


def test_to_dag_first_occurrence(oracle):
    """toDAG (structure.h:703-763): unique items keep first-occurrence order; lossless."""
    import tdag
    dense = blocky_grid(32, 1)
    tree = tdag.EditStructure.from_svo_bytes(oracle.svo_from_dense(dense))
    dag = tdag.EditStructure.from_svo_bytes(oracle.to_dag(oracle.svo_from_dense(dense)))
    assert dag.structure_type == 1
    # first-occurrence order of leaves
    seen = {}
    for m in tree.sub_grids:
        seen.setdefault(int(m), len(seen))
    assert [int(v) for v in dag.sub_grids] == list(seen.keys())
    for z in range(0, 32, 3):
        for y in range(0, 32, 5):
            for x in range(32):
                assert svo_get(dag, x, y, z) == bool(dense[z, y, x])


CFGS = [(1, 1, 1, 4), (1, 1, 0, 4), (1, 0, 1, 3), (0, 1, 1, 2), (0, 0, 1, 4), (0, 0, 0, 0)]


@pytest.mark.parametrize("cfg", CFGS)
@pytest.mark.parametrize("kind", ["terrain", "blocky", "random"])
def test_oracle_tdag_is_lossless(oracle, cfg, kind):
    """The decoded Transform DAG reproduces every voxel (the reference's verifyComplexTransformDAG
    self-check, transform_dag_encoding.h:81-117)."""
    from oracle import generator
    dense = {"terrain": lambda: generator.terrain(64, 4), "blocky": lambda: blocky_grid(64, 2),
             "random": lambda: random_grid(32, 0.1, 5)}[kind]()
    svo = dag_svo_bytes(oracle, dense)
    tdag_bytes, stats, _ = oracle.construct_tdag(svo, *cfg)
    dec = oracle.tdag_decode(tdag_bytes, dense.shape[0])
    assert np.array_equal(dec, dense)
    if cfg[2]:
        assert stats["verifications"] >= stats["verified"] > 0


def test_encode_fixed64_roundtrip(oracle):
    import tdag
    rng = np.random.default_rng(0)
    for level in (2, 3, 4):
        R = 1 << level
        for _ in range(200):
            ptr = int(rng.integers(0, 1 << 30))
            sym = tuple(bool(b) for b in rng.integers(0, 2, 3))
            perm = tdag.PERMUTATIONS[int(rng.integers(0, 6))]
            t = tuple(int(v) for v in rng.integers(-(R - 1), R, 3))
            v = tdag.tp_create(ptr, sym, perm, t)
            e = oracle.encode_fixed64(v, level)
            assert e == tdag.encode_fixed64(v, level)
            assert oracle.decode_fixed64(e, level) == v


def test_transform_group_laws(oracle):
    c, inv, pos = oracle.transform_tables()
    assert all(c[0, a] == a and c[a, 0] == a for a in range(48))
    for a in range(48):
        assert c[a, inv[a]] == 0 and c[inv[a], a] == 0
        assert sorted(pos[a]) == list(range(8))
    rng = np.random.default_rng(1)
    for _ in range(500):
        a, b, d = (int(x) for x in rng.integers(0, 48, 3))
        assert c[c[a, b], d] == c[a, c[b, d]]
        for i in range(8):  # composition acts on positions
            assert pos[c[a, b], i] == pos[a, pos[b, i]]


def test_find_duplicates_self_consistency(oracle):
    """Every non-unique item is reconstructed exactly by its parent's transform."""
    import tdag
    rng = np.random.default_rng(3)
    level, R = 3, 8
    base = rng.random((40, R, R, R)) < 0.2
    items = [base[i] for i in range(40)]
    for i in range(40):
        sh = np.zeros_like(base[i])  # clipped shift: z + 1, x - 1, then mirror y
        sh[1:, :, :-1] = base[i][:-1, :, 1:]
        items.append(sh[:, ::-1, :])
    dense = np.stack(items)
    grids = np.packbits(dense.reshape(len(items), -1).astype(np.uint8), axis=1, bitorder="little").view(np.uint64)
    mapping, uniq, st = oracle.find_duplicates(level, grids)
    assert len(uniq) < len(items)
    kept = {int(u): k for k, u in enumerate(uniq)}
    for i, m in enumerate(mapping):
        ptr, sym, perm, t = tdag.tp_decode(int(m))
        if i in kept:
            assert ptr == kept[i] and not any(sym) and perm == (0, 1, 2) and t == (0, 0, 0)
            continue
        src = dense[int(uniq[ptr])]  # [z, y, x]
        xyz = np.transpose(src, (2, 1, 0))  # [x, y, z]
        p = np.zeros_like(xyz)
        idx = np.argwhere(xyz)
        for (x, y, z) in idx:
            v = (x, y, z)
            w = [v[perm[0]], v[perm[1]], v[perm[2]]]
            for k in range(3):
                if sym[k]:
                    w[k] = R - 1 - w[k]
                w[k] += t[k]
            if all(0 <= w[k] < R for k in range(3)):
                p[w[0], w[1], w[2]] = 1
        assert np.array_equal(np.transpose(p, (2, 1, 0)), dense[i])


@pytest.mark.parametrize("sym,axis", [(1, 1), (1, 0), (0, 1)])
@pytest.mark.parametrize("kind", ["terrain", "blocky"])
def test_hierarchical_equals_build_without_translation(oracle, sym, axis, kind):
    """constructTransformDAGHierarchical (transform_dag_hierarchical.cpp:304-529) is the construction
    with translation off: the library's tdag_build_hierarchical runs tdag_build with translation 0,
    whose bytes the GPU parity tests compare with construct_tdag(..., translation=0)."""
    from oracle import generator
    dense = {"terrain": lambda: generator.terrain(64, 3), "blocky": lambda: blocky_grid(64, 4)}[kind]()
    svo = dag_svo_bytes(oracle, dense)
    full, _, _ = oracle.construct_tdag(svo, sym, axis, 0, 0)
    assert full[:-8] == oracle.hierarchical(svo, sym, axis)  # .tdag = structure + 8-byte config
