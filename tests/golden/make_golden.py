"""Writes tests/golden/golden.json: SHA-256 digests and sizes of the oracle's outputs on fixed inputs.

Each case records the `.svo` input, the oracle's `.tdag` (constructTransformDAG, default config) and
its `.tdag16` encodings (pointer tables + Huffman, and plain; canonical tie order). The library must
reproduce every digest byte for byte (tests/test_gpu_golden.py); tests/test_golden_cpu.py re-derives
the small cases with the oracle.

Cases:
  terrain256  the 256^3 terrain workload: oracle/generator.py terrain(256, seed 1) -> SVO -> toDAG.
  scene2048   the bench grid: the device-generated 2048^3 primitive scene
              (SceneSpec(PRIMITIVES, 2048, seed 1, 4000 primitives)), as an .svo file written by
              tdag.scene_svdag(...).to_host().to_svo_bytes(); pass its path with --scene2048.

Usage: python tests/golden/make_golden.py [--scene2048 path/to/scene2048.svo]
"""
import argparse
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import generator  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def digest(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def case(svo: bytes) -> dict:
    t0 = time.time()
    tdag, stats, _ = orc.construct_tdag(svo)
    t1 = time.time()
    out = {"svo_sha256": digest(svo), "svo_bytes": len(svo), "tdag_sha256": digest(tdag), "tdag_bytes": len(tdag),
           "oracle_build_s": round(t1 - t0, 1), "oracle_threads": orc.max_threads(), "unique_translation": stats["unique"]}
    for name, pt, hf in (("tdag16_tables_huffman", True, True), ("tdag16_plain", False, False)):
        data, lv = orc.encode_tdag16(tdag, pointer_tables=pt, huffman=hf, tie=orc.TIE_CANONICAL)
        out[name + "_sha256"] = digest(data)
        out[name + "_bytes"] = len(data)
        out[name + "_nodes"] = [l["num_nodes"] for l in lv]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene2048", default="")
    args = ap.parse_args()
    path = os.path.join(HERE, "golden.json")
    golden = json.load(open(path)) if os.path.exists(path) else {}
    dense = generator.terrain(256, 1)
    golden["terrain256"] = dict(case(orc.to_dag(orc.svo_from_dense(dense))), input="oracle/generator.py terrain(256, seed=1), SVO -> toDAG")
    if args.scene2048:
        svo = open(args.scene2048, "rb").read()
        golden["scene2048"] = dict(case(svo), input="tdag.scene_svdag(SceneSpec(kind=PRIMITIVES, resolution=2048, seed=1, num_primitives=4000), to_dag=True)")
    json.dump(golden, open(path, "w"), indent=1, sort_keys=True)
    print(json.dumps(golden, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
