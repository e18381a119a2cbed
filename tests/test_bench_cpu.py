"""Host-side pieces of bench.py's JSON line, on CPU: the cost models behind `roofline`, the workload
description in `config`, and the lookups of the measured peak and the recorded DRAM traffic."""
import argparse
import json
import os

import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def bench():
    import sys
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import bench as b
    return b


def _args(**kw):
    a = dict(resolution=2048, primitives=4000, seed=1, scene="primitives")
    a.update(kw)
    return argparse.Namespace(**a)


def test_search_model_bytes(bench):
    # M * G + P * 16: one R^3 grid per source item, one 16-byte slot per non-empty box
    st = {"items": 1000, "probes": 50_000}
    assert bench.search_model_bytes(4, st) == 1000 * 512 + 50_000 * 16
    assert bench.search_model_bytes(3, st) == 1000 * 64 + 50_000 * 16
    assert bench.search_model_bytes(2, st) == 1000 * 8 + 50_000 * 16


def test_probe_dram_bytes(bench):
    # grids in, three line orientations out (3 R^2 u16), one 16-byte record per filter survivor
    st = {"items": 10, "filter_pass": 7}
    assert bench.probe_algorithmic_bytes(4, st) == 10 * 512 + 10 * 3 * 256 * 2 + 7 * 16


def test_build_model_bytes(bench):
    st = {"hierarchical": {"2": {"items": 100, "unique": 40}, "3": {"items": 30, "unique": 20}},
          "translation": {"4": {"items": 5, "probes": 9, "verifications": 2}}}
    want = (100 * (8 + 16) + 40 * 8) + (30 * (32 + 8 * 16 + 16) + 20 * 64)
    want += 5 * (512 + 8 * 16 + 8) + 9 * 16 + 2 * 2 * 512 + 5 * 8
    assert bench.build_model_bytes(st) == want


def test_workload_config(bench):
    cfg = bench.workload_config(_args(), voxels=102_614_527)
    assert cfg["resolution"] == 2048 and cfg["primitives"] == 4000 and cfg["scene"] == "primitives"
    assert cfg["solid_voxels"] == 102_614_527
    assert "2048^3 primitive-union shell" in cfg["workload"] and "flushed" in cfg["l2"]
    t = bench.workload_config(_args(scene="terrain", resolution=256))
    assert t["primitives"] == 0 and "256^3 solid fBm terrain" in t["workload"] and "solid_voxels" not in t


def test_recorded_traffic_is_per_workload(bench):
    p = os.path.join(REPO, "profiles", "probe_traffic.json")
    with open(p) as f:
        rec = json.load(f)["workloads"]
    key = "primitives/2048/4000/1"
    assert bench.load_traffic(4, _args()) == rec[key]["4"]
    # another workload has no capture: no traffic figure rather than a borrowed one
    assert bench.load_traffic(4, _args(resolution=4096, primitives=12000)) is None
    assert bench.load_traffic(3, _args()) == rec[key].get("3")


def test_peak_source(bench):
    peak, kind = bench.load_peaks()
    assert peak > 0
    assert kind == ("measured" if os.path.exists(os.path.join(REPO, "MEASURED_PEAKS.json")) else "fallback")


def test_cpu_samples_are_restrictions_of_the_grid(bench, oracle):
    """The reference arm's per-step inputs: distinct seeded sub-volumes, each the SVDAG of the grid's
    restriction to its box (checked against the whole 128^3 grid)."""
    import numpy as np
    args = _args(resolution=128, primitives=60, sample_resolution=32)
    samples = bench.cpu_samples(args, 5)
    full = oracle.scene_dense(128, 1, 60)
    origins = [o for _, _, o in samples]
    assert len(set(origins)) == 5
    for svo, vox, (x, y, z) in samples:
        sub = full[z:z + 32, y:y + 32, x:x + 32]
        assert vox == int(sub.sum()) > 0
        assert svo == oracle.to_dag(oracle.svo_from_dense(sub))


def test_reference_arm_runs_without_the_product_library(tmp_path):
    """--impl reference prints its JSON line and never loads libtdag.so."""
    import subprocess
    import sys
    code = ("import runpy, sys; sys.argv=['bench.py','--impl','reference','--steps','2','--warmup','1','--resolution','128',"
            "'--primitives','60','--sample-resolution','32']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('LOADED', [m for m in open('/proc/self/maps').read().split() if m.endswith('.so') and 'libtdag' in m])")
    r = subprocess.run([sys.executable, "-c", code], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    line = json.loads(lines[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert "LOADED []" in r.stdout
