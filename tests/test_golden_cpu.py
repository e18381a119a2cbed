"""The oracle against the committed golden digests (tests/golden/golden.json, written by
tests/golden/make_golden.py): the config-0 terrain case is re-derived here on every run."""
import hashlib
import json
import os

import pytest

from conftest import REPO

GOLDEN = json.load(open(os.path.join(REPO, "tests", "golden", "golden.json")))


def _d(b):
    return hashlib.sha256(b).hexdigest()


def test_oracle_reproduces_terrain256_golden(oracle):
    from oracle import generator
    g = GOLDEN["terrain256"]
    svo = oracle.to_dag(oracle.svo_from_dense(generator.terrain(256, 1)))
    assert _d(svo) == g["svo_sha256"]
    tdag, _, _ = oracle.construct_tdag(svo)
    assert _d(tdag) == g["tdag_sha256"]
    for name, pt, hf in (("tdag16_tables_huffman", True, True), ("tdag16_plain", False, False)):
        data, _ = oracle.encode_tdag16(tdag, pointer_tables=pt, huffman=hf)
        assert _d(data) == g[name + "_sha256"], name


def test_golden_file_covers_the_bench_grid():
    g = GOLDEN.get("scene2048")
    assert g is not None and len(g["tdag_sha256"]) == 64 and g["svo_bytes"] > 0
