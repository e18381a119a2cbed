"""GPU tests of the input side: SVO build (A1), toDAG (A2) and the procedural scenes (N1)."""
import numpy as np
import pytest

from helpers import blocky_grid, random_grid

pytestmark = pytest.mark.gpu


def _svo_struct(tdaglib, oracle, dense, dag):
    svo = oracle.svo_from_dense(dense)
    if dag:
        svo = oracle.to_dag(svo)
    return tdaglib.EditStructure.from_svo_bytes(svo)


def _assert_same(a, b):
    assert a.resolution == b.resolution and a.root_level == b.root_level
    assert a.structure_type == b.structure_type
    assert np.array_equal(a.sub_grids, b.sub_grids)
    for la, lb in zip(a.nodes_per_level, b.nodes_per_level):
        assert np.array_equal(la, lb)


@pytest.mark.parametrize("dag", [False, True])
@pytest.mark.parametrize("kind", ["random", "blocky", "terrain", "empty", "full"])
def test_svo_and_todag_match_oracle(oracle, tdaglib, gpu_ctx, kind, dag):
    from oracle import generator
    dense = {"random": lambda: random_grid(32, 0.05, 1), "blocky": lambda: blocky_grid(64, 3),
             "terrain": lambda: generator.terrain(64, 2), "empty": lambda: np.zeros((16, 16, 16), np.uint8),
             "full": lambda: np.ones((32, 32, 32), np.uint8)}[kind]()
    ref = _svo_struct(tdaglib, oracle, dense, dag)
    g = tdaglib.svdag_from_dense(dense, to_dag=dag, ctx=gpu_ctx)
    got = g.to_host()
    _assert_same(got, ref)
    assert g.voxel_count == int(dense.sum())


@pytest.mark.parametrize("res,seed", [(64, 1), (128, 5)])
def test_terrain_scene_matches_cpu_generator(oracle, tdaglib, gpu_ctx, res, seed):
    from oracle import generator
    dense = generator.terrain(res, seed)
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_TERRAIN, resolution=res, seed=seed, shell=False)
    got = tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx)
    _assert_same(got.to_host(), _svo_struct(tdaglib, oracle, dense, True))
    assert got.voxel_count == int(dense.sum())


@pytest.mark.parametrize("res,n,seed,shell", [(64, 40, 3, True), (128, 120, 7, True), (128, 60, 9, False)])
def test_primitive_scene_matches_cpu_generator(oracle, tdaglib, gpu_ctx, res, n, seed, shell):
    from oracle import generator
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=res, seed=seed, num_primitives=n, copy_percent=30, shell=shell)
    prims = tdaglib.scene_primitives(spec)
    dense = generator.primitives_scene(res, prims, shell=shell)
    got = tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx)
    _assert_same(got.to_host(), _svo_struct(tdaglib, oracle, dense, True))
    assert got.voxel_count == int(dense.sum())


def test_scene_build_end_to_end_matches_oracle(oracle, tdaglib, gpu_ctx):
    """Device scene -> device SVDAG -> device TDAG equals the oracle's TDAG of the same SVDAG."""
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=128, seed=11, num_primitives=150)
    g = tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx)
    host = g.to_host()
    ref, _, _ = oracle.construct_tdag(host.to_svo_bytes())
    cfg = tdaglib.TransformDAGConfig()
    got = tdaglib.write_tdag(tdaglib.construct_transform_dag(host, cfg, ctx=gpu_ctx), cfg)
    assert got == ref


@pytest.mark.parametrize("res,chunk,n,seed,kind", [(256, 64, 200, 3, "primitives"), (512, 128, 600, 8, "primitives"), (256, 128, 50, 4, "primitives"),
                                                   (128, 64, 0, 2, "terrain")])
def test_chunked_scene_equals_single_pass(tdaglib, gpu_ctx, res, chunk, n, seed, kind):
    """The chunked generator (chunk SVOs merged into global first-occurrence tables) builds the same
    SVDAG as the single-pass generator: same items, same order, same voxel count."""
    k = tdaglib.SCENE_PRIMITIVES if kind == "primitives" else tdaglib.SCENE_TERRAIN
    base = dict(kind=k, resolution=res, seed=seed, num_primitives=n, shell=kind == "primitives")
    one = tdaglib.scene_svdag(tdaglib.SceneSpec(**base), to_dag=True, ctx=gpu_ctx)
    many = tdaglib.scene_svdag(tdaglib.SceneSpec(**base, chunk_resolution=chunk), to_dag=True, ctx=gpu_ctx)
    _assert_same(many.to_host(), one.to_host())
    assert many.voxel_count == one.voxel_count


@pytest.mark.parametrize("slabs", [1, 40])
def test_chunked_scene_with_a_tiny_slab_pool(tdaglib, gpu_ctx, slabs):
    """The global slab hash tables of the chunked generator start with a pool of 1 or 40 spare slabs,
    so their chains exhaust it again and again (TDAG_ERR_ALLOC on the device, never a spin); the host
    doubles the pool and resumes each insertion. The SVDAG is the single-pass one all the same."""
    base = dict(kind=tdaglib.SCENE_PRIMITIVES, resolution=512, seed=9, num_primitives=300)
    one = tdaglib.scene_svdag(tdaglib.SceneSpec(**base), to_dag=True, ctx=gpu_ctx)
    ctx = tdaglib.Context(tuning={"slab_pool_slabs": slabs})
    try:
        many = tdaglib.scene_svdag(tdaglib.SceneSpec(**base, chunk_resolution=64), to_dag=True, ctx=ctx)
        _assert_same(many.to_host(), one.to_host())
        assert many.voxel_count == one.voxel_count
    finally:
        ctx.close()


def _covered_bricks(res, prims):
    """32^3 bricks whose 34^3 halo box lies inside one box or ball primitive and inside the grid."""
    from oracle.generator import PERMS
    n = 0
    for bz in range(res // 32):
        for by in range(res // 32):
            for bx in range(res // 32):
                lo = [bx * 32 - 1, by * 32 - 1, bz * 32 - 1]
                if min(lo) < 0 or max(lo) + 34 > res:
                    continue
                for p in prims:
                    ext = [p["size"][PERMS[p["xform"] & 7][k]] for k in range(3)]
                    if p["type"] == 0 and all(p["offset"][k] <= lo[k] and lo[k] + 34 <= p["offset"][k] + ext[k] for k in range(3)):
                        n += 1
                        break
                    if p["type"] == 1:
                        r = p["radius"]
                        c = [p["offset"][k] + r for k in range(3)]
                        if all(sum((lo[k] + (33 if (m >> k) & 1 else 0) - c[k]) ** 2 for k in range(3)) <= r * r for m in range(8)):
                            n += 1
                            break
    return n


@pytest.mark.parametrize("shell", [True, False])
def test_scene_with_solid_bricks_matches_cpu_generator(oracle, tdaglib, gpu_ctx, shell):
    """Large primitives: bricks entirely inside one primitive take the generator's solid-brick exit."""
    from oracle import generator
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=512, seed=21, num_primitives=60, copy_percent=30, shell=shell)
    prims = tdaglib.scene_primitives(spec)
    assert _covered_bricks(512, prims) > 0
    dense = generator.primitives_scene(512, prims, shell=shell)
    got = tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx)
    _assert_same(got.to_host(), _svo_struct(tdaglib, oracle, dense, True))
    assert got.voxel_count == int(dense.sum())


def test_device_scene_equals_cpu_scene_statement(oracle, tdaglib, gpu_ctx):
    """The device generator and the C++ CPU statement (oracle/scene_oracle.cpp, which builds the CPU
    baseline's inputs) agree on a 512^3 primitive scene, and a CPU sub-box equals the device grid's
    subtree at that box."""
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=512, seed=13, num_primitives=400)
    got = tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx).to_host()
    dense = oracle.scene_dense(512, 13, 400)
    _assert_same(got, _svo_struct(tdaglib, oracle, dense, True))
    sub = oracle.scene_dense(512, 13, 400, origin=(256, 128, 0), size=128)
    assert np.array_equal(sub, dense[0:128, 128:256, 256:384])


def test_streamed_scene_resumes_from_its_checkpoints(tdaglib, gpu_ctx, tmp_path):
    """A streamed scene build stopped twice on the host (TDAG_ERR_INTERRUPTED after a given number
    of chunks, checkpoint written) and resumed from its checkpoint file ends with the SVDAG of an
    uninterrupted build: same items, same order, same voxel count. A checkpoint of another scene or a
    truncated one is refused (TDAG_ERR_CORRUPT), never read past its end."""
    from tdag import _abi
    base = dict(kind=tdaglib.SCENE_PRIMITIVES, resolution=512, seed=5, num_primitives=300, chunk_resolution=64)
    whole = tdaglib.scene_svdag(tdaglib.SceneSpec(**base), to_dag=True, ctx=gpu_ctx)
    path = str(tmp_path / "scene.ckpt")
    for stop in (70, 150):
        with pytest.raises(tdaglib.TDagError) as e:
            tdaglib.scene_svdag_checkpointed(tdaglib.SceneSpec(**base), path, every_chunks=16, stop_after_chunks=stop, ctx=gpu_ctx)
        assert e.value.code == _abi.TDAG_ERR_INTERRUPTED
    saved = open(path, "rb").read()
    resumed = tdaglib.scene_svdag_checkpointed(tdaglib.SceneSpec(**base), path, every_chunks=16, ctx=gpu_ctx)
    _assert_same(resumed.to_host(), whole.to_host())
    assert resumed.voxel_count == whole.voxel_count
    # the same file for another scene, and a truncated copy
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.scene_svdag_checkpointed(tdaglib.SceneSpec(**dict(base, seed=6)), path, ctx=gpu_ctx)
    assert e.value.code == _abi.TDAG_ERR_CORRUPT
    cut = str(tmp_path / "cut.ckpt")
    open(cut, "wb").write(saved[: len(saved) // 2])
    with pytest.raises(tdaglib.TDagError) as e:
        tdaglib.scene_svdag_checkpointed(tdaglib.SceneSpec(**base), cut, ctx=gpu_ctx)
    assert e.value.code == _abi.TDAG_ERR_CORRUPT
