"""Autotuner for batched Transform-DAG builds.

Sweeps the knobs of libtdag.so's tdag_tuning on a given batch:

* ``table_load_percent`` — the corner-hash table's load factor (50-85 %);
* ``filter_bits_per_key`` — the membership filter's density;
* ``search_ctas_per_sm`` — persistent probe CTAs per SM (the probe kernel's block shape);
* ``probe_bulk_copy`` — the level-4 probe's source staging (bulk copy or cooperative loads);
* ``verify_lanes`` — threads per exact subgrid verification in the lookup (1, 4, 8 or 32);
* ``lookup_tile`` — probe records a lookup warp claims at a time (the work tile, 32-1024).

Every configuration must give the same result (the build is exact, so a difference is a bug and
raises). Timings are the library's own CUDA-event device times. ``mode="descent"`` (the default)
tunes one knob at a time, keeping the best value of each before the next, for up to ``passes``
rounds; ``mode="grid"`` times the whole product of the space.
"""
from __future__ import annotations

import hashlib
import itertools
from typing import Dict, List, Optional, Sequence, Tuple

import tdag

# 0 keeps the library's own choice: for filter_bits_per_key 32 bits per key unless the filter would
# pass 32 MB, for search_ctas_per_sm as many probe CTAs as fit an SM, for probe_bulk_copy cooperative loads
DEFAULT_SPACE = {
    "table_load_percent": (50, 60, 70, 85),
    "filter_bits_per_key": (0, 8, 16, 32),
    "search_ctas_per_sm": (0, 2, 3, 4),
    "probe_bulk_copy": (0, 1),
    "verify_lanes": (32, 1, 4, 8),
    "lookup_tile": (32, 64, 128, 256, 512, 1024),
}
# where the descent starts: the library's defaults
DEFAULT_START = {"table_load_percent": 50, "filter_bits_per_key": 0, "search_ctas_per_sm": 0, "probe_bulk_copy": 0,
                 "verify_lanes": 32, "lookup_tile": 32}


def result_digest(structures: Sequence[tdag.EditStructure]) -> str:
    h = hashlib.sha256()
    for s in structures:
        h.update(s.to_bytes())
    return h.hexdigest()


def autotune_batched(dags: List["tdag.DeviceSvdag"], config: tdag.TransformDAGConfig, device: int = 0,
                     space: Optional[Dict[str, Tuple[int, ...]]] = None, repeats: int = 1, mode: str = "descent",
                     passes: int = 2, start: Optional[Dict[str, int]] = None):
    """Returns (best tuning dict, best device ms, list of (tuning, ms) for every configuration timed)."""
    space = space or DEFAULT_SPACE
    keys = list(space)
    table: List[Tuple[dict, float]] = []
    timed: Dict[tuple, float] = {}
    ref = {"digest": None}

    def measure(tuning: dict) -> float:
        sig = tuple(sorted(tuning.items()))
        if sig in timed:
            return timed[sig]
        ctx = tdag.Context(device, tuning)
        ms = float("inf")
        digest = None
        try:
            for _ in range(repeats):
                results, stats = tdag.construct_transform_dag_batched_device(dags, config, ctx=ctx)
                ms = min(ms, stats["total_ms"])
                if digest is None:
                    digest = result_digest([r.to_host(ctx) for r in results])
                for r in results:
                    r.free()
        finally:
            ctx.close()
        if ref["digest"] is None:
            ref["digest"] = digest
        elif digest != ref["digest"]:
            raise RuntimeError(f"tuning {tuning} changed the result; the build must be exact for every tuning")
        timed[sig] = ms
        table.append((dict(tuning), ms))
        return ms

    if mode == "grid":
        best = (None, float("inf"))
        for values in itertools.product(*(space[k] for k in keys)):
            tuning = dict(zip(keys, values))
            ms = measure(tuning)
            if ms < best[1]:
                best = (tuning, ms)
        return best[0], best[1], table
    if mode != "descent":
        raise ValueError(f"unknown autotune mode {mode!r}")
    cur = {k: (start or DEFAULT_START).get(k, space[k][0]) for k in keys}
    best_ms = measure(cur)
    for _ in range(max(passes, 1)):
        improved = False
        for k in keys:
            for v in space[k]:
                if v == cur[k]:
                    continue
                trial = dict(cur, **{k: v})
                ms = measure(trial)
                if ms < best_ms:
                    cur, best_ms, improved = trial, ms, True
        if not improved:
            break
    return cur, best_ms, table
