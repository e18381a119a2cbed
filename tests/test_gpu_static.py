"""GPU parity of constructStaticTransformDAG (tdag_build_static) with the oracle, byte for byte."""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid

pytestmark = pytest.mark.gpu

CASES = [
    ("blocky64", lambda g: blocky_grid(64, 3)),
    ("blocky128", lambda g: blocky_grid(128, 9)),
    ("terrain256", lambda g: g.terrain(256, 1)),
    ("random32", lambda g: random_grid(32, 0.2, 4)),
]
CFGS = [(1, 1, 1, 4), (1, 1, 0, 4), (1, 0, 1, 3), (0, 0, 0, 0)]


@pytest.mark.parametrize("cfg", CFGS)
@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_static_build_matches_oracle(oracle, tdaglib, gpu_ctx, name, make, cfg):
    from oracle import generator
    svo = dag_svo_bytes(oracle, make(generator))
    static_in = oracle.to_static(svo)
    ref = oracle.construct_static_tdag(static_in, *cfg)
    c = tdaglib.TransformDAGConfig(bool(cfg[0]), bool(cfg[1]), bool(cfg[2]), cfg[3])
    got = tdaglib.construct_static_transform_dag(tdaglib.StaticStructure.from_bytes(static_in), c, ctx=gpu_ctx)
    assert got.to_bytes() == ref


def test_static_build_rejects_unreferenced_words(tdaglib, gpu_ctx, oracle):
    """A level holding a node no parent references is rejected (TDAG_ERR_CORRUPT), not misread."""
    st = tdaglib.StaticStructure.from_bytes(oracle.to_static(dag_svo_bytes(oracle, blocky_grid(64, 3))))
    extra = st.words[4][:2].copy()  # a header and one child word copied to the end of level 4
    st.words[4] = np.concatenate([st.words[4], extra])
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.construct_static_transform_dag(st, ctx=gpu_ctx)
    assert e.value.code == 6


def test_static_tdag_encodes_to_tdag16(oracle, tdaglib, gpu_ctx):
    """constructTransformDAG16 of a static transform DAG: the encoder on the unpacked structure, equal
    to the oracle's encoding of it and lossless."""
    dense = blocky_grid(128, 9)
    st_bytes = oracle.construct_static_tdag(oracle.to_static(dag_svo_bytes(oracle, dense)))
    st = tdaglib.StaticStructure.from_bytes(st_bytes, "transform")
    cfg = tdaglib.TransformDAGConfig()
    for pt, hf in [(False, False), (True, True)]:
        got = tdaglib.construct_transform_dag16(st, cfg, tdaglib.TransformEncodingConfig(pt, hf), ctx=gpu_ctx)
        want, _ = oracle.encode_tdag16(tdaglib.write_tdag(st.to_edit(), cfg), pointer_tables=pt, huffman=hf)
        assert got == want
        assert np.array_equal(oracle.decode_tdag16(got, 128), dense)
