"""CPU tests of the StaticStructure path (constructStaticTransformDAG, transform_dag.cpp:242-390):
the packed layout (structure.h:765-798) against the oracle's restatement, lossless decoding of the
oracle's static transform DAG, and its relation to the EditStructure path."""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid

CASES = [("blocky64", lambda: blocky_grid(64, 3)), ("random32", lambda: random_grid(32, 0.2, 4)), ("blocky128", lambda: blocky_grid(128, 9))]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_static_layout_matches_oracle(oracle, name, make):
    import tdag
    svo = dag_svo_bytes(oracle, make())
    ref = oracle.to_static(svo)
    st = tdag.StaticStructure.from_edit(tdag.EditStructure.from_svo_bytes(svo))
    assert st.to_bytes() == ref
    assert tdag.StaticStructure.from_bytes(ref).to_bytes() == ref


@pytest.mark.parametrize("cfg", [dict(), dict(translation=False), dict(max_level=3), dict(symmetry=False, axis=False, translation=False)])
@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_static_tdag_is_lossless_and_agrees_below_the_boundary(oracle, name, make, cfg):
    import tdag
    dense = make()
    svo = dag_svo_bytes(oracle, dense)
    args = (cfg.get("symmetry", True), cfg.get("axis", True), cfg.get("translation", True), cfg.get("max_level", 4))
    st = oracle.construct_static_tdag(oracle.to_static(svo), *args)
    assert np.array_equal(oracle.static_tdag_decode(st, dense.shape[0]), dense)
    # the EditStructure path makes the same decisions: identical packed levels up to the translation
    # levels (both keep referenced nodes in input order there), same node counts above
    edit, _ = tdag.read_tdag(oracle.construct_tdag(svo, *args)[0])
    packed_edit = tdag.StaticStructure.from_edit(edit)
    got = tdag.StaticStructure.from_bytes(st, "transform")
    assert np.array_equal(got.sub_grids, packed_edit.sub_grids)
    top = args[3] if args[2] else 2
    for l in range(3, got.root_level + 1):
        assert got.words[l].shape == packed_edit.words[l].shape
        if l <= top:
            assert np.array_equal(got.words[l], packed_edit.words[l]), l


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_static_unpacks_to_the_same_structure(oracle, name, make):
    """StaticStructure -> EditStructure: the inverse of the packing, for u32 inputs and for the static
    transform DAG (which then equals the oracle's own unpacking, byte for byte)."""
    import tdag
    svo = dag_svo_bytes(oracle, make())
    edit = tdag.EditStructure.from_svo_bytes(svo)
    back = tdag.StaticStructure.from_bytes(oracle.to_static(svo)).to_edit()
    assert back.to_bytes() == edit.to_bytes()
    st = tdag.StaticStructure.from_bytes(oracle.construct_static_tdag(oracle.to_static(svo)), "transform")
    assert tdag.StaticStructure.from_edit(st.to_edit()).to_bytes() == st.to_bytes()
