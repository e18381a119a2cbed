"""The CPU restatement pinned against the reference's own code.

``oracle/_ref/libtdag_ref.so`` is the reference's Transform-DAG path compiled from its own sources
(find_translation.cpp, transform_dag.cpp, transform_dag_hierarchical.cpp, structure.h,
transform_dag_encoding.cpp, huffman.cpp) by ``oracle/ref.mk``. Every case compares the oracle's bytes
with the reference's bytes on the same input: the .svo (EditStructure(VoxelGrid)), toDAG, the .tdag
for every config flag combination and translation level, the hierarchical pass alone, the static
structure path, and the .tdag16 in all four encodings (libstdc++ tie order; the reference's
uninitialised struct padding masked). The library is compared with the oracle by the GPU tests.

The reference's sources exist only in the development container, so these tests skip elsewhere;
tests/golden/golden.json carries reference-made digests to every machine (test_golden_cpu.py).
"""
import numpy as np
import pytest

from helpers import blocky_grid, mask_tdag16_padding, random_grid

ref = pytest.importorskip("oracle.reference")

pytestmark = pytest.mark.skipif(not (ref.sources_present() or ref.available()),
                                reason="the reference's sources (and so oracle/_ref) are not on this machine")

CONFIGS = [(1, 1, 1, 4), (1, 0, 1, 4), (0, 1, 1, 4), (1, 1, 0, 4), (0, 0, 1, 4), (0, 0, 0, 4), (1, 1, 1, 3), (1, 1, 1, 2)]


def _grids():
    from oracle import generator
    return {
        "terrain64": generator.terrain(64, 3),
        "blocky64": blocky_grid(64, 7),
        "random64": random_grid(64, 0.03, 11),
        "primitives64": generator.primitives_scene(64, _prims(64, 5)),
    }


def _prims(res, seed):
    rng = np.random.default_rng(seed)
    prims = []
    for i in range(10):
        t = int(rng.integers(0, 3))
        if i > 2 and rng.random() < 0.4:
            p = dict(prims[int(rng.integers(0, i))])
            p["xform"] = int(rng.integers(0, 6)) | (int(rng.integers(0, 8)) << 3)
        else:
            s = int(rng.integers(4, res // 2))
            p = {"type": t, "size": [s, s, s] if t else [int(v) for v in rng.integers(3, res // 2, 3)],
                 "radius": (s - 1) // 2, "seed": int(rng.integers(1, 1 << 31)), "xform": 0}
            if t == 1:
                p["size"] = [2 * p["radius"] + 1] * 3
        ext = max(p["size"])
        p["offset"] = [int(v) for v in rng.integers(0, max(1, res - ext), 3)]
        prims.append(p)
    return prims


@pytest.fixture(scope="module")
def reflib():
    ref.build()
    ref.lib()
    return ref


@pytest.fixture(scope="module")
def grids():
    return _grids()


@pytest.mark.parametrize("name", ["terrain64", "blocky64", "random64", "primitives64"])
def test_svo_and_todag_equal_reference(reflib, oracle, grids, name):
    dense = grids[name]
    svo = reflib.svo_from_dense(dense)
    assert oracle.svo_from_dense(dense) == svo
    assert oracle.to_dag(svo) == reflib.to_dag(svo)


@pytest.mark.parametrize("name", ["terrain64", "blocky64", "random64", "primitives64"])
@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "s{}p{}t{}L{}".format(*c))
def test_transform_dag_equals_reference(reflib, oracle, grids, name, cfg):
    dag = reflib.to_dag(reflib.svo_from_dense(grids[name]))
    want = reflib.construct_tdag(dag, *cfg)
    got, _, _ = oracle.construct_tdag(dag, *cfg)
    assert got == want


@pytest.mark.parametrize("name", ["terrain64", "blocky64"])
@pytest.mark.parametrize("sym,axis", [(1, 1), (1, 0), (0, 1)])
def test_hierarchical_equals_reference(reflib, oracle, grids, name, sym, axis):
    dag = reflib.to_dag(reflib.svo_from_dense(grids[name]))
    assert oracle.hierarchical(dag, bool(sym), bool(axis)) == reflib.hierarchical(dag, sym, axis)


@pytest.mark.parametrize("name", ["terrain64", "blocky64", "random64"])
def test_static_path_equals_reference(reflib, oracle, grids, name):
    dag = reflib.to_dag(reflib.svo_from_dense(grids[name]))
    st = reflib.to_static(dag)
    assert oracle.to_static(dag) == st
    for cfg in ((1, 1, 1, 4), (1, 0, 1, 3)):
        assert oracle.construct_static_tdag(st, *cfg) == reflib.construct_static_tdag(st, *cfg)


@pytest.mark.parametrize("name", ["terrain64", "blocky64", "random64", "primitives64"])
@pytest.mark.parametrize("pt,hf", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_tdag16_equals_reference(reflib, oracle, grids, name, pt, hf):
    dag = reflib.to_dag(reflib.svo_from_dense(grids[name]))
    tdag = reflib.construct_tdag(dag)
    want = mask_tdag16_padding(reflib.encode_tdag16(tdag, pt, hf))
    got, _ = oracle.encode_tdag16(tdag, pointer_tables=bool(pt), huffman=bool(hf), tie=oracle.TIE_LIBSTDCXX)
    assert got == mask_tdag16_padding(got), "the oracle writes zero padding"
    assert got == want


def test_terrain128_end_to_end_equals_reference(reflib, oracle):
    from oracle import generator
    dense = generator.terrain(128, 1)
    dag = reflib.to_dag(reflib.svo_from_dense(dense))
    tdag = reflib.construct_tdag(dag)
    got, _, _ = oracle.construct_tdag(oracle.to_dag(oracle.svo_from_dense(dense)))
    assert got == tdag
    for pt, hf in ((0, 0), (1, 1)):
        enc, _ = oracle.encode_tdag16(got, pointer_tables=bool(pt), huffman=bool(hf), tie=oracle.TIE_LIBSTDCXX)
        assert enc == mask_tdag16_padding(reflib.encode_tdag16(tdag, pt, hf))


@pytest.mark.parametrize("pt,hf", [(0, 0), (1, 1)])
def test_static_tdag16_equals_reference(reflib, oracle, grids, pt, hf):
    """constructTransformDAG16 of a static transform DAG (transform_dag_encoding.cpp:519-697) makes the
    same bytes as the encoder of the unpacked structure, which is how the library encodes it."""
    import tdag
    dag = reflib.to_dag(reflib.svo_from_dense(grids["blocky64"]))
    st = reflib.construct_static_tdag(reflib.to_static(dag))
    edit = tdag.write_tdag(tdag.StaticStructure.from_bytes(st, "transform").to_edit(), tdag.TransformDAGConfig())
    got, _ = oracle.encode_tdag16(edit, pointer_tables=bool(pt), huffman=bool(hf), tie=oracle.TIE_LIBSTDCXX)
    assert got == mask_tdag16_padding(reflib.encode_static_tdag16(st, pointer_tables=pt, huffman=hf))
