"""The level-4 probe kernel with its source grids staged by 1-D bulk copies (cp.async.bulk through
the TMA unit, one source ahead, completed on mbarriers with bounded waits) gives the same results as
with cooperative loads: full builds compared byte for byte with the oracle."""
import pytest

from helpers import blocky_grid, dag_svo_bytes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [1, 2])
def test_bulk_copy_staging_is_exact(oracle, tdaglib, mode):
    from oracle import generator
    ctx = tdaglib.Context(tuning={"probe_bulk_copy": mode})
    try:
        for dense, cfg in ((blocky_grid(128, 31), {}), (generator.terrain(128, 5), {"translation": True}),
                           (blocky_grid(64, 32), {"symmetry": False})):
            svo = dag_svo_bytes(oracle, dense)
            c = tdaglib.TransformDAGConfig(symmetry=cfg.get("symmetry", True))
            want, _, _ = oracle.construct_tdag(svo, c.symmetry, c.axis_permutation, c.translation, c.max_translation_level)
            got = tdaglib.write_tdag(tdaglib.construct_transform_dag(tdaglib.EditStructure.from_svo_bytes(svo), c, ctx=ctx), c)
            assert got == want
        spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=512, seed=3, num_primitives=300)
        sv = tdaglib.scene_svdag(spec, to_dag=True, ctx=ctx)
        want, _, _ = oracle.construct_tdag(sv.to_host().to_svo_bytes())
        cfg = tdaglib.TransformDAGConfig()
        assert tdaglib.write_tdag(tdaglib.construct_transform_dag_device(sv, cfg, ctx=ctx).to_host(ctx), cfg) == want
    finally:
        ctx.close()
