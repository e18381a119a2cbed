"""Full-size parity against the committed golden digests (tests/golden/golden.json): the library's
.svo, .tdag and .tdag16 bytes of the config-0 terrain and of the 2048^3 bench grid must equal the
oracle's, digest for digest. The 2048^3 digests were computed by the oracle on the same SVDAG
(tests/golden/make_golden.py), so this checks the whole pipeline bit for bit at the bench size."""
import hashlib
import json
import os

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(REPO, "tests", "golden", "golden.json")))


def _d(b):
    return hashlib.sha256(b).hexdigest()


def _check(tdaglib, gpu_ctx, g, sv):
    assert _d(sv.to_host().to_svo_bytes()) == g["svo_sha256"]
    cfg = tdaglib.TransformDAGConfig()
    dev = tdaglib.construct_transform_dag_device(sv, cfg, ctx=gpu_ctx)
    assert _d(tdaglib.write_tdag(dev.to_host(gpu_ctx), cfg)) == g["tdag_sha256"]
    for name, pt, hf in (("tdag16_tables_huffman", True, True), ("tdag16_plain", False, False)):
        data = tdaglib.construct_transform_dag16(dev, cfg, tdaglib.TransformEncodingConfig(pt, hf), ctx=gpu_ctx)
        assert _d(data) == g[name + "_sha256"], name


def test_terrain256_matches_golden(tdaglib, gpu_ctx):
    from oracle import generator
    sv = tdaglib.svdag_from_dense(generator.terrain(256, 1), ctx=gpu_ctx)
    _check(tdaglib, gpu_ctx, GOLDEN["terrain256"], sv)


def test_bench_grid_2048_matches_golden(tdaglib, gpu_ctx):
    spec = tdaglib.SceneSpec(kind=tdaglib.SCENE_PRIMITIVES, resolution=2048, seed=1, num_primitives=4000)
    sv = tdaglib.scene_svdag(spec, to_dag=True, ctx=gpu_ctx)
    _check(tdaglib, gpu_ctx, GOLDEN["scene2048"], sv)
