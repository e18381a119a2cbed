"""Batched build (tdag_build_batched): every result equals the single-grid build and the oracle."""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes, random_grid

pytestmark = pytest.mark.gpu


def _inputs(oracle, tdaglib):
    from oracle import generator
    grids = [generator.terrain(64, 3), blocky_grid(32, 4), random_grid(32, 0.05, 9), blocky_grid(64, 8), generator.terrain(32, 5),
             blocky_grid(128, 2, n_boxes=20)]
    svos = [dag_svo_bytes(oracle, g) for g in grids]
    return svos, [tdaglib.EditStructure.from_svo_bytes(s) for s in svos]


@pytest.mark.parametrize("cfgt", [(1, 1, 1, 4), (1, 1, 0, 4), (0, 1, 1, 3)])
def test_batched_equals_single_and_oracle(oracle, tdaglib, gpu_ctx, cfgt):
    svos, dags = _inputs(oracle, tdaglib)
    cfg = tdaglib.TransformDAGConfig(*[bool(v) for v in cfgt[:3]], cfgt[3])
    batch = tdaglib.construct_transform_dag_batched(dags, cfg, ctx=gpu_ctx)
    assert len(batch) == len(dags)
    for svo, d, b in zip(svos, dags, batch):
        single = tdaglib.construct_transform_dag(d, cfg, ctx=gpu_ctx)
        got = tdaglib.write_tdag(b, cfg)
        assert got == tdaglib.write_tdag(single, cfg)
        ref, _, _ = oracle.construct_tdag(svo, *cfgt)
        assert got == ref


def test_batched_device_scenes(oracle, tdaglib, gpu_ctx):
    """Device-generated scenes of different sizes through the device batch entry point."""
    specs = [tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=r, seed=s, num_primitives=n)
             for r, s, n in ((64, 1, 30), (128, 2, 80), (64, 3, 10), (32, 4, 8))]
    devs = [tdaglib.scene_svdag(sp, to_dag=True, ctx=gpu_ctx) for sp in specs]
    cfg = tdaglib.TransformDAGConfig()
    results, stats = tdaglib.construct_transform_dag_batched_device(devs, cfg, ctx=gpu_ctx)
    assert stats["kernel_launches"] > 0
    for dv, r in zip(devs, results):
        host = dv.to_host()
        single = tdaglib.construct_transform_dag_device(dv, cfg, ctx=gpu_ctx)
        # compare the device results through their node counts and the host path's bytes
        ref, _, _ = oracle.construct_tdag(host.to_svo_bytes())
        rs, _ = tdaglib.read_tdag(ref)
        rc = r._rp.contents
        assert rc.leaf_count == len(rs.sub_grids)
        for lvl in range(3, host.root_level + 1):
            assert rc.node_counts[lvl] == len(rs.nodes_per_level[lvl])
        single.free()
        r.free()
