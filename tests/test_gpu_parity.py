"""GPU parity: libtdag.so (through its C ABI) against the CPU oracle, bit for bit."""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid, structure_from_svo

pytestmark = pytest.mark.gpu


def _gpu_tdag_bytes(tdaglib, gpu_ctx, svo, cfg):
    dag = structure_from_svo(tdaglib, svo)
    out = tdaglib.construct_transform_dag(dag, cfg, ctx=gpu_ctx)
    return tdaglib.write_tdag(out, cfg)


CASES = [
    ("terrain32", lambda g: g.terrain(32, 7)),
    ("terrain64", lambda g: g.terrain(64, 1)),
    ("blocky32", lambda g: blocky_grid(32, 3)),
    ("blocky64", lambda g: blocky_grid(64, 5)),
    ("random32_sparse", lambda g: random_grid(32, 0.03, 11)),
    ("random32_dense", lambda g: random_grid(32, 0.6, 12)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_construct_transform_dag_matches_oracle(oracle, tdaglib, gpu_ctx, name, make):
    from oracle import generator
    dense = make(generator)
    svo = dag_svo_bytes(oracle, dense)
    cfg = tdaglib.TransformDAGConfig()
    ref, _, _ = oracle.construct_tdag(svo, True, True, True, 4)
    got = _gpu_tdag_bytes(tdaglib, gpu_ctx, svo, cfg)
    assert got == ref


@pytest.mark.parametrize("sym,axis,trans,maxl", [(1, 1, 0, 4), (1, 0, 1, 4), (0, 1, 1, 3), (0, 0, 1, 2), (0, 0, 0, 0), (1, 1, 1, 3)])
def test_config_variants(oracle, tdaglib, gpu_ctx, sym, axis, trans, maxl):
    dense = blocky_grid(64, 9)
    svo = dag_svo_bytes(oracle, dense)
    cfg = tdaglib.TransformDAGConfig(bool(sym), bool(axis), bool(trans), maxl)
    ref, _, _ = oracle.construct_tdag(svo, sym, axis, trans, maxl)
    got = _gpu_tdag_bytes(tdaglib, gpu_ctx, svo, cfg)
    assert got == ref


def test_config0_terrain256(oracle, tdaglib, gpu_ctx):
    from oracle import generator
    dense = generator.terrain(256, 1)
    svo = dag_svo_bytes(oracle, dense)
    ref, st, _ = oracle.construct_tdag(svo)
    got = _gpu_tdag_bytes(tdaglib, gpu_ctx, svo, tdaglib.TransformDAGConfig())
    assert got == ref


@pytest.mark.parametrize("level", [2, 3, 4])
def test_find_duplicates_level(oracle, tdaglib, gpu_ctx, level):
    rng = np.random.default_rng(level)
    R = 1 << level
    W = R ** 3 // 64
    # sparse random grids plus shifted/mirrored copies of a few of them
    n = 300
    grids = np.zeros((n, W), np.uint64)
    dense = (rng.random((n, R, R, R)) < 0.15)
    for i in range(60, n):
        src = dense[rng.integers(0, 60)]
        sh = rng.integers(-2, 3, size=3)
        cp = np.roll(src, tuple(sh), axis=(0, 1, 2))
        if rng.random() < 0.5:
            cp = cp[::-1]
        if rng.random() < 0.5:
            cp = np.transpose(cp, (1, 0, 2))
        dense[i] = cp
    flat = dense.reshape(n, -1)  # [z, y, x] -> bit x + R*y + R*R*z
    bits = np.packbits(flat.astype(np.uint8), axis=1, bitorder="little")
    grids = bits.view(np.uint64).reshape(n, W)
    m_ref, u_ref, _ = oracle.find_duplicates(level, grids)
    u_got, m_got = tdaglib.find_duplicates_among_flattened_items(level, grids, ctx=gpu_ctx)
    assert np.array_equal(u_ref, u_got)
    assert np.array_equal(m_ref, m_got)


def _level_grids(level, n=300, seed=None):
    rng = np.random.default_rng(level if seed is None else seed)
    R = 1 << level
    W = R ** 3 // 64
    dense = (rng.random((n, R, R, R)) < 0.15)
    for i in range(60, n):
        src = dense[rng.integers(0, 60)]
        cp = np.roll(src, tuple(rng.integers(-2, 3, size=3)), axis=(0, 1, 2))
        if rng.random() < 0.5:
            cp = cp[::-1]
        if rng.random() < 0.5:
            cp = np.transpose(cp, (1, 0, 2))
        dense[i] = cp
    bits = np.packbits(dense.reshape(n, -1).astype(np.uint8), axis=1, bitorder="little")
    return bits.view(np.uint64).reshape(n, W)


@pytest.mark.parametrize("lanes,tile", [(1, 32), (4, 64), (8, 256), (32, 1024), (4, 1024)])
@pytest.mark.parametrize("level", [2, 3, 4])
def test_verify_lanes_and_lookup_tile(oracle, tdaglib, level, lanes, tile):
    """Every verification width (threads per subgrid) and lookup claim size gives the oracle's result."""
    grids = _level_grids(level, seed=100 + level)
    m_ref, u_ref, _ = oracle.find_duplicates(level, grids)
    ctx = tdaglib.Context(0, {"verify_lanes": lanes, "lookup_tile": tile})
    try:
        u_got, m_got = tdaglib.find_duplicates_among_flattened_items(level, grids, ctx=ctx)
        assert np.array_equal(u_ref, u_got) and np.array_equal(m_ref, m_got)
        # and a whole build through the same context
        dense = blocky_grid(64, 9)
        svo = dag_svo_bytes(oracle, dense)
        ref, _, _ = oracle.construct_tdag(svo)
        assert _gpu_tdag_bytes(tdaglib, ctx, svo, tdaglib.TransformDAGConfig()) == ref
    finally:
        ctx.close()


@pytest.mark.parametrize("knob,value", [("verify_lanes", 2), ("verify_lanes", 64), ("lookup_tile", 48), ("lookup_tile", 2048)])
def test_bad_lookup_knobs_are_rejected(tdaglib, knob, value):
    grids = _level_grids(3, n=100)
    ctx = tdaglib.Context(0, {knob: value})
    try:
        with pytest.raises(tdaglib.TDagError) as e:
            tdaglib.find_duplicates_among_flattened_items(3, grids, ctx=ctx)
        assert e.value.code == 1  # TDAG_ERR_ARG
    finally:
        ctx.close()
