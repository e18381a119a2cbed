"""The CPU statement of the procedural scenes (oracle/scene_oracle.cpp) against the library's host
primitive list and against the numpy statement (oracle/generator.py). The device generator is checked
against both by tests/test_gpu_scene.py. Together they let the CPU baseline build its inputs without
the product library."""
import numpy as np
import pytest


@pytest.mark.parametrize("res,count,seed", [(64, 20, 1), (256, 200, 2), (2048, 4000, 1), (16384, 60000, 1)])
def test_primitive_list_equals_library(oracle, tdaglib, res, count, seed):
    got = oracle.scene_primitives(res, seed, count)
    want = tdaglib.scene_primitives(tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=res, seed=seed, num_primitives=count))
    assert len(got) == len(want) == count
    for g, w in zip(got, want):
        assert (int(g["type"]), int(g["xform"]), tuple(int(v) for v in g["size"]), int(g["radius"]),
                tuple(int(v) for v in g["offset"]), int(g["seed"]), int(g["source"])) == \
               (w["type"], w["xform"], tuple(w["size"]), w["radius"], tuple(w["offset"]), w["seed"], w["source"])


def _as_dicts(prims):
    return [{"type": int(p["type"]), "xform": int(p["xform"]), "size": [int(v) for v in p["size"]], "radius": int(p["radius"]),
             "offset": [int(v) for v in p["offset"]], "seed": int(p["seed"])} for p in prims]


@pytest.mark.parametrize("res,count,seed", [(64, 20, 1), (64, 40, 5), (128, 60, 3)])
def test_dense_scene_equals_numpy_statement(oracle, res, count, seed):
    prims = oracle.scene_primitives(res, seed, count)
    from oracle import generator
    for shell in (True, False):
        want = generator.primitives_scene(res, _as_dicts(prims), shell=shell)
        got = oracle.scene_dense(res, seed, count, shell=shell)
        assert np.array_equal(got, want), shell


def test_sub_box_is_the_restriction_of_the_grid(oracle):
    full = oracle.scene_dense(128, 4, 50)
    for origin in ((0, 0, 0), (64, 0, 32), (32, 96, 64)):
        sub = oracle.scene_dense(128, 4, 50, origin=origin, size=32)
        x, y, z = origin
        assert np.array_equal(sub, full[z:z + 32, y:y + 32, x:x + 32]), origin
