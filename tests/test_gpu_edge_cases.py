"""Degenerate and extreme inputs through the whole GPU pipeline, against the oracle byte for byte:
empty grids, single voxels in both corners, a full solid grid, a checkerboard (every leaf the same,
no two neighbours alike), stripes, and the smallest grid a translation level allows."""
import numpy as np
import pytest

from helpers import dag_svo_bytes

pytestmark = pytest.mark.gpu


def _cases():
    z, y, x = np.indices((32, 32, 32))
    c = {}
    c["empty32"] = np.zeros((32, 32, 32), np.uint8)
    v = np.zeros((32, 32, 32), np.uint8)
    v[0, 0, 0] = 1
    c["voxel_at_origin"] = v
    v = np.zeros((64, 64, 64), np.uint8)
    v[63, 63, 63] = 1
    c["voxel_at_far_corner"] = v
    c["full64"] = np.ones((64, 64, 64), np.uint8)
    c["checker32"] = ((x + y + z) % 2).astype(np.uint8)
    c["stripes32"] = ((x // 3) % 2).astype(np.uint8)
    c["diagonal32"] = (x == y).astype(np.uint8) & (y == z).astype(np.uint8)
    return c


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_case_matches_oracle(oracle, tdaglib, gpu_ctx, name):
    dense = CASES[name]
    svo = dag_svo_bytes(oracle, dense)
    ref, _, _ = oracle.construct_tdag(svo)
    cfg = tdaglib.TransformDAGConfig()
    host = tdaglib.EditStructure.from_svo_bytes(svo)
    got = tdaglib.write_tdag(tdaglib.construct_transform_dag(host, cfg, ctx=gpu_ctx), cfg)
    assert got == ref
    # the device SVO builder and the .tdag16 encoder on the same input
    sv = tdaglib.svdag_from_dense(dense, ctx=gpu_ctx)
    assert sv.to_host().to_svo_bytes() == svo
    for pt, hf in [(False, False), (True, True)]:
        data = tdaglib.construct_transform_dag16(tdaglib.read_tdag(ref)[0], cfg, tdaglib.TransformEncodingConfig(pt, hf), ctx=gpu_ctx)
        want, _ = oracle.encode_tdag16(ref, pointer_tables=pt, huffman=hf)
        assert data == want
        assert np.array_equal(oracle.decode_tdag16(data, dense.shape[0]), dense)


def test_smallest_grid_for_each_translation_level(oracle, tdaglib, gpu_ctx):
    """The root must lie above the highest translation level: 16^3 works with levels up to 3 and is
    rejected with level 4 (the reference would index past its levels; here TDAG_ERR_ARG)."""
    dense = np.zeros((16, 16, 16), np.uint8)
    dense[4:8, 4:9, 3:8] = 1
    dense[12, 1, 9] = 1
    svo = dag_svo_bytes(oracle, dense)
    host = tdaglib.EditStructure.from_svo_bytes(svo)
    for maxl in (2, 3):
        cfg = tdaglib.TransformDAGConfig(max_translation_level=maxl)
        ref, _, _ = oracle.construct_tdag(svo, max_level=maxl)
        assert tdaglib.write_tdag(tdaglib.construct_transform_dag(host, cfg, ctx=gpu_ctx), cfg) == ref
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.construct_transform_dag(host, tdaglib.TransformDAGConfig(max_translation_level=4), ctx=gpu_ctx)
    assert e.value.code == 1
