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


def _scene_batch(tdaglib, gpu_ctx):
    specs = [tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=r, seed=s, num_primitives=n)
             for r, s, n in ((64, 11, 30), (128, 12, 80), (32, 13, 8), (64, 14, 10), (128, 15, 40))]
    return [tdaglib.scene_svdag(sp, to_dag=True, ctx=gpu_ctx) for sp in specs]


@pytest.mark.parametrize("cfgt", [(1, 1, 1, 4), (1, 1, 0, 4), (0, 1, 1, 3)])
def test_batch_graph_equals_eager_batch_and_oracle(oracle, tdaglib, gpu_ctx, cfgt):
    """The batched build captured in one CUDA graph (tdag_batch_graph_*): two launches in a row, each
    result equal bit for bit to the eager batched build's and to the oracle's."""
    devs = _scene_batch(tdaglib, gpu_ctx)
    cfg = tdaglib.TransformDAGConfig(*[bool(v) for v in cfgt[:3]], cfgt[3])
    eager, _ = tdaglib.construct_transform_dag_batched_device(devs, cfg, ctx=gpu_ctx)
    want = [tdaglib.write_tdag(r.to_host(gpu_ctx), cfg) for r in eager]
    for r in eager:
        r.free()
    for dv, w in zip(devs, want):
        ref, _, _ = oracle.construct_tdag(dv.to_host().to_svo_bytes(), *cfgt)
        assert w == ref
    graph = tdaglib.BatchGraph(devs, cfg, ctx=gpu_ctx)
    for launch in range(2):
        results, stats = graph.launch()
        assert stats["kernel_launches"] > 0 and stats["total_ms"] > 0, f"launch {launch}"
        for i, r in enumerate(results):
            assert tdaglib.write_tdag(r.to_host(gpu_ctx), cfg) == want[i], f"launch {launch}, grid {i}"
            r.free()
    graph.free()


def test_batch_graph_rejects_a_changed_batch(tdaglib, gpu_ctx):
    """A launch on a batch whose arrays changed since the graph was made returns TDAG_ERR_ARG without
    running the graph; with the contents restored the graph runs again."""
    import ctypes
    import torch
    from tdag import _abi

    devs = _scene_batch(tdaglib, gpu_ctx)[:3]
    cfg = tdaglib.TransformDAGConfig()
    graph = tdaglib.BatchGraph(devs, cfg, ctx=gpu_ctx)
    first, _ = graph.launch()
    want = [tdaglib.write_tdag(r.to_host(gpu_ctx), cfg) for r in first]
    L = tdaglib.lib()
    va, vb = devs[0].view(), devs[1].view()
    leaves_a = devs[0].to_host().sub_grids
    leaves_b = devs[1].to_host().sub_grids
    k = next(i for i in range(min(len(leaves_a), len(leaves_b))) if leaves_a[i] != leaves_b[i])
    a_word = ctypes.cast(va.leaves, ctypes.c_void_p).value + 8 * k
    b_word = ctypes.cast(vb.leaves, ctypes.c_void_p).value + 8 * k
    saved = torch.empty(1, dtype=torch.int64, device=torch.device("cuda", gpu_ctx.device))
    _abi.check(L.tdag_device_copy(gpu_ctx.handle, saved.data_ptr(), a_word, 8))
    _abi.check(L.tdag_device_copy(gpu_ctx.handle, a_word, b_word, 8))  # grid 0's leaf k now differs
    with pytest.raises(_abi.TDagError) as e:
        graph.launch()
    assert e.value.code == _abi.TDAG_ERR_ARG
    _abi.check(L.tdag_device_copy(gpu_ctx.handle, a_word, saved.data_ptr(), 8))
    again, _ = graph.launch()
    assert [tdaglib.write_tdag(r.to_host(gpu_ctx), cfg) for r in again] == want
    graph.free()


def test_autotune_on_a_small_batch(oracle, tdaglib, gpu_ctx):
    """The autotuner times every configuration it tries on the device (each one's bytes checked
    against the first's) and its choice builds the oracle's bytes."""
    from tdag import autotune

    devs = _scene_batch(tdaglib, gpu_ctx)[:3]
    cfg = tdaglib.TransformDAGConfig()
    space = {"table_load_percent": (50, 85), "verify_lanes": (1, 4, 8, 32), "lookup_tile": (32, 256, 1024)}
    best, ms, table = autotune.autotune_batched(devs, cfg, device=gpu_ctx.device, space=space)
    assert set(best) == set(space) and ms > 0 and len(table) >= 6
    ctx = tdaglib.Context(gpu_ctx.device, best)
    try:
        results, _ = tdaglib.construct_transform_dag_batched_device(devs, cfg, ctx=ctx)
        for dv, r in zip(devs, results):
            ref, _, _ = oracle.construct_tdag(dv.to_host().to_svo_bytes())
            assert tdaglib.write_tdag(r.to_host(ctx), cfg) == ref
            r.free()
    finally:
        ctx.close()


def test_batch_graph_replays_class_table_regrows(oracle, tdaglib):
    """Class tables started far too small (400 % load) fill up, report TDAG_ERR_TABLE_FULL and are
    regrown; whether a table is full depends only on its number of distinct classes, so the graph
    replays the same failed attempts and retries as its plan and still builds the oracle's bytes."""
    ctx = tdaglib.Context(tuning={"class_table_load_percent": 400})
    try:
        devs = _scene_batch(tdaglib, ctx)[:3]
        cfg = tdaglib.TransformDAGConfig()
        graph = tdaglib.BatchGraph(devs, cfg, ctx=ctx)
        for _ in range(2):
            results, _ = graph.launch()
            for dv, r in zip(devs, results):
                ref, _, _ = oracle.construct_tdag(dv.to_host().to_svo_bytes())
                assert tdaglib.write_tdag(r.to_host(ctx), cfg) == ref
                r.free()
        graph.free()
    finally:
        ctx.close()
