"""Failure detection and recovery on the GPU, without faulting, trapping or hanging it.

Device code never spins unbounded and never traps (the reference's cuckoo insert and slab allocator
retry without a bound: find_translation.cu:780-783, dynamic_slab_alloc.h:74-115). A full table is a
status word the host reads after the stage; an allocation past the context's budget is refused on the
host. These tests provoke both through tdag_tuning and check what the caller sees:

* class tables started far too small (class_table_load_percent 400) fill up, the host doubles them
  and reruns the pass, and the result is byte-identical to the oracle's;
* with the regrow limit exhausted the call returns TDAG_ERR_TABLE_FULL;
* a device-memory limit below what a build needs returns TDAG_ERR_OOM;
* a dangling child index in the input returns TDAG_ERR_CORRUPT;
and after each failure a fresh call on the same GPU succeeds and is exact.
"""
import numpy as np
import pytest

from helpers import blocky_grid, dag_svo_bytes

pytestmark = pytest.mark.gpu

TABLE_FULL, OOM, CORRUPT = 3, 2, 6


@pytest.fixture(scope="module")
def case(oracle):
    dense = blocky_grid(64, 21)
    svo = dag_svo_bytes(oracle, dense)
    ref, _, _ = oracle.construct_tdag(svo)
    return dense, svo, ref


def _build(tdaglib, ctx, svo):
    dag = tdaglib.EditStructure.from_svo_bytes(svo)
    cfg = tdaglib.TransformDAGConfig()
    out, stats = tdaglib.construct_transform_dag(dag, cfg, ctx=ctx, return_stats=True)
    return tdaglib.write_tdag(out, cfg), stats


def test_full_class_tables_are_regrown_with_identical_output(tdaglib, case):
    dense, svo, ref = case
    ctx = tdaglib.Context(tuning={"class_table_load_percent": 400})
    try:
        got, stats = _build(tdaglib, ctx, svo)
        assert got == ref
        assert stats["table_regrows"] >= 1  # a table of a quarter of the items' slots cannot hold every class
        # toDAG's class tables take the same path
        sv = tdaglib.svdag_from_dense(dense, ctx=ctx)
        assert sv.to_host().to_svo_bytes() == svo
    finally:
        ctx.close()


def test_table_full_past_the_regrow_limit_is_reported(tdaglib, gpu_ctx, case):
    dense, svo, ref = case
    ctx = tdaglib.Context(tuning={"class_table_load_percent": 100000, "table_regrow_limit": 1})
    try:
        with pytest.raises(tdaglib.TDagError) as e:
            _build(tdaglib, ctx, svo)
        assert e.value.code == TABLE_FULL
        assert "regrow" in str(e.value)
    finally:
        ctx.close()
    assert _build(tdaglib, gpu_ctx, svo)[0] == ref


def test_device_memory_limit_reports_oom(tdaglib, gpu_ctx, case):
    dense, svo, ref = case
    ctx = tdaglib.Context(tuning={"device_memory_limit": 64 << 10})
    try:
        with pytest.raises(tdaglib.TDagError) as e:
            _build(tdaglib, ctx, svo)
        assert e.value.code == OOM
        assert "limit" in str(e.value)
        # the failed call released what it held: a second attempt fails the same way, not worse
        with pytest.raises(tdaglib.TDagError) as e2:
            _build(tdaglib, ctx, svo)
        assert e2.value.code == OOM
    finally:
        ctx.close()
    roomy = tdaglib.Context(tuning={"device_memory_limit": 8 << 30})
    try:
        assert _build(tdaglib, roomy, svo)[0] == ref
        assert _build(tdaglib, roomy, svo)[0] == ref  # the budget is returned after every build
    finally:
        roomy.close()


def test_dangling_child_index_is_reported(tdaglib, gpu_ctx, case):
    dense, svo, ref = case
    dag = tdaglib.EditStructure.from_svo_bytes(svo)
    lvl = 3
    nodes = dag.nodes_per_level[lvl]
    row, col = np.argwhere(nodes != 0xFFFFFFFF)[0]
    nodes[row, col] = len(dag.sub_grids) + 5
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.construct_transform_dag(dag, tdaglib.TransformDAGConfig(), ctx=gpu_ctx)
    assert e.value.code == CORRUPT
    assert _build(tdaglib, gpu_ctx, svo)[0] == ref
