"""Writes tests/golden/golden.json: SHA-256 digests and sizes of outputs on fixed inputs.

Each case records the `.svo` input, the `.tdag` (constructTransformDAG, default config) and the
`.tdag16` encodings. Two sources of digests:

* ``reference``: the reference's own code, compiled from its sources into oracle/_ref
  (oracle/ref.mk, oracle/reference.py). Written where the reference's sources exist. Its `.tdag16`
  digests are taken with the bytes the reference leaves uninitialised set to zero (struct padding:
  byte 3 of TransformDAGConfig, the last 4 bytes of each 16-byte Huffman `Code`), which is what the
  library and the oracle write.
* the oracle (oracle/oracle.py): the same digests, plus the `.tdag16` in the canonical tie order.

tests/test_golden_cpu.py re-derives the small cases with the oracle and requires them to equal the
reference's digests; tests/test_gpu_golden.py requires the library to reproduce them.

Cases:
  terrain256  the 256^3 terrain workload: oracle/generator.py terrain(256, seed 1) -> SVO -> toDAG.
  blocky128   tests/helpers.py blocky_grid(128, seed 3): boxes with mirrored and permuted copies.
  scene2048   the bench grid: the device-generated 2048^3 primitive scene
              (SceneSpec(PRIMITIVES, 2048, seed 1, 4000 primitives)), as an .svo file written by
              tdag.scene_svdag(...).to_host().to_svo_bytes(); pass its path with --scene2048.
              Its reference digests are added by --scene2048-reference (a serial build of hours).

Usage: python tests/golden/make_golden.py [--scene2048 path.svo [--scene2048-reference]]
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
sys.path.insert(0, os.path.join(REPO, "tests"))

from helpers import blocky_grid, mask_tdag16_padding  # noqa: E402
from oracle import generator  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import reference as ref  # noqa: E402

ENCODINGS = (("tdag16_tables_huffman", True, True), ("tdag16_plain", False, False),
             ("tdag16_tables", True, False), ("tdag16_huffman", False, True))
VARIANTS = ((1, 0, 1, 4), (0, 1, 1, 4), (1, 1, 0, 4), (1, 1, 1, 3))


def digest(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def vname(v):
    return "s{}p{}t{}L{}".format(*v)


def oracle_case(svo: bytes) -> dict:
    t0 = time.time()
    tdag, stats, _ = orc.construct_tdag(svo)
    t1 = time.time()
    out = {"svo_sha256": digest(svo), "svo_bytes": len(svo), "tdag_sha256": digest(tdag), "tdag_bytes": len(tdag),
           "oracle_build_s": round(t1 - t0, 1), "oracle_threads": orc.max_threads(), "unique_translation": stats["unique"]}
    for name, pt, hf in ENCODINGS:
        data, lv = orc.encode_tdag16(tdag, pointer_tables=pt, huffman=hf, tie=orc.TIE_LIBSTDCXX)
        out[name + "_sha256"] = digest(data)
        out[name + "_bytes"] = len(data)
        out[name + "_nodes"] = [l["num_nodes"] for l in lv]
        canon, _ = orc.encode_tdag16(tdag, pointer_tables=pt, huffman=hf, tie=orc.TIE_CANONICAL)
        out[name + "_canonical_sha256"] = digest(canon)
    return out


def reference_case(svo: bytes, variants=VARIANTS) -> dict:
    t0 = time.time()
    tdag = ref.construct_tdag(svo)
    t1 = time.time()
    out = {"svo_sha256": digest(svo), "tdag_sha256": digest(tdag), "reference_build_s": round(t1 - t0, 1),
           "reference_threads": 1}
    for name, pt, hf in ENCODINGS:
        out[name + "_sha256"] = digest(mask_tdag16_padding(ref.encode_tdag16(tdag, pt, hf)))
    out["tdag_variants_sha256"] = {vname(v): digest(ref.construct_tdag(svo, *v)) for v in variants}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene2048", default="")
    ap.add_argument("--scene2048-reference", action="store_true")
    ap.add_argument("--keep-small", action="store_true", help="keep the small cases' digests as they are")
    ap.add_argument("--reuse-oracle", action="store_true", help="keep scene2048's oracle digests when its .svo is unchanged")
    args = ap.parse_args()
    path = os.path.join(HERE, "golden.json")
    golden = json.load(open(path)) if os.path.exists(path) else {}
    have_ref = ref.sources_present() or ref.available()
    if have_ref:
        ref.build()
    small = {
        "terrain256": (generator.terrain(256, 1), "oracle/generator.py terrain(256, seed=1), SVO -> toDAG"),
        "blocky128": (blocky_grid(128, 3), "tests/helpers.py blocky_grid(128, seed=3), SVO -> toDAG"),
    }
    for key, (dense, what) in ([] if args.keep_small else small.items()):
        svo = orc.to_dag(orc.svo_from_dense(dense))
        g = dict(oracle_case(svo), input=what)
        if have_ref:
            rsvo = ref.to_dag(ref.svo_from_dense(dense))
            g["reference"] = reference_case(rsvo)
        elif "reference" in golden.get(key, {}):
            g["reference"] = golden[key]["reference"]
        golden[key] = g
    if args.scene2048:
        svo = open(args.scene2048, "rb").read()
        old = golden.get("scene2048", {})
        if args.reuse_oracle and old.get("svo_sha256") == digest(svo) and "tdag16_plain_canonical_sha256" in old:
            g = {k: v for k, v in old.items() if k != "reference"}
        else:
            g = dict(oracle_case(svo), input="tdag.scene_svdag(SceneSpec(kind=PRIMITIVES, resolution=2048, seed=1, num_primitives=4000), to_dag=True)")
        if args.scene2048_reference and have_ref:
            g["reference"] = reference_case(svo, variants=())
        elif "reference" in golden.get("scene2048", {}):
            g["reference"] = golden["scene2048"]["reference"]
        golden["scene2048"] = g
    json.dump(golden, open(path, "w"), indent=1, sort_keys=True)
    print(json.dumps(golden, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
