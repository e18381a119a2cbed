"""Autotuner for batched Transform-DAG builds.

Sweeps the knobs of libtdag.so's tdag_tuning — the corner-hash table load factor (50-85 %), the
membership filter density (bits per distinct key), the number of persistent probe CTAs per SM and the
level-4 probe's source staging (bulk copy or cooperative loads) — on a given
batch, checks that every configuration gives the same result (the build is exact, so any difference
is a bug), and returns the fastest. Timings are the library's own CUDA-event device times.
"""
from __future__ import annotations

import hashlib
import itertools
from typing import Dict, List, Optional, Sequence, Tuple

import tdag

DEFAULT_SPACE = {
    "table_load_percent": (50, 70, 85),
    "filter_bits_per_key": (16, 32),
    "search_ctas_per_sm": (3, 4),
    "probe_bulk_copy": (1, 2),
}


def result_digest(structures: Sequence[tdag.EditStructure]) -> str:
    h = hashlib.sha256()
    for s in structures:
        h.update(s.to_bytes())
    return h.hexdigest()


def autotune_batched(dags: List["tdag.DeviceSvdag"], config: tdag.TransformDAGConfig, device: int = 0,
                     space: Optional[Dict[str, Tuple[int, ...]]] = None, repeats: int = 1):
    """Returns (best tuning dict, best device ms, list of (tuning, ms) for every candidate)."""
    space = space or DEFAULT_SPACE
    keys = list(space)
    table = []
    ref_digest = None
    best = (None, float("inf"))
    for values in itertools.product(*(space[k] for k in keys)):
        tuning = dict(zip(keys, values))
        ctx = tdag.Context(device, tuning)
        ms = float("inf")
        digest = None
        for _ in range(repeats):
            results, stats = tdag.construct_transform_dag_batched_device(dags, config, ctx=ctx)
            ms = min(ms, stats["total_ms"])
            if digest is None:
                digest = result_digest([r.to_host(ctx) for r in results])
            for r in results:
                r.free()
        ctx.close()
        if ref_digest is None:
            ref_digest = digest
        elif digest != ref_digest:
            raise RuntimeError(f"tuning {tuning} changed the result; the build must be exact for every tuning")
        table.append((tuning, ms))
        if ms < best[1]:
            best = (tuning, ms)
    return best[0], best[1], table
