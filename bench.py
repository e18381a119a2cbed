"""Benchmark: Transform-DAG construction throughput (Mvoxels/s) on GB300.

Workload (one step = one constructTransformDAG over one SVDAG): the 2048^3 single-grid build,
exhaustive symmetry + axis permutation + translation matching at the reference's default window
(maxTranslationLevel 4). The grid is a seeded union of 4,000 boxes / spheres / fBm terrain blocks,
30% of them mirrored, axis-permuted or translated copies of earlier ones, reduced to its 1-voxel
surface shell, generated on the device (synthetic data; the reference's mesh scenes are not
available). SVO build and toDAG happen once before timing.

value   : solid input voxels / device time of the build, input and output resident in HBM.
e2e     : the same through tdag_build() with pinned host buffers: host->device copy of the SVDAG,
          the build, and the device->host copy of the Transform DAG inside the timed region.
roofline: the dominant kernel -- the translation probe kernel of the level with the largest probe
          time -- with the algorithmic bytes of the search's cost model (M*G + P*16: one grid per source,
          one 16-byte slot per non-empty probe) over its CUDA-event device time, against
          MEASURED_PEAKS.json. Beside it: the DRAM-only bytes; its filter loads per second against this
          GPU's random-load ceiling for L2-resident buffers (tdag_l2_probe_peak), the resource that
          actually bounds it; and the whole build's model bytes over the build time.
cpu_baseline: the CPU oracle (the restatement of the reference's CPU path, pinned byte for byte to
          the reference's own code; all host threads) on the WHOLE grid, once, in a child process with
          a time limit (--cpu-baseline full, the default for the single-grid workload); its key
          "sample" adds the same oracle on seeded random sub-volumes, as the reference arm runs it.
--impl reference: the same oracle on a different seeded random aligned sub-volume of the same grid
          per step (256^3 by default), generated on the CPU by oracle/scene_oracle.cpp, so that this
          arm loads no product library.

Multi-GPU: the path does not shard; --gpus N runs N independent replicas (one per rank), and value
is the sum of their throughputs (max-over-ranks timing).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "i3d2025-voxel-transform-dag_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "TDAG build Mvoxels/s"
UNIT = "Mvoxels/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--resolution", type=int, default=2048)
    ap.add_argument("--primitives", type=int, default=4000)
    ap.add_argument("--scene", default="primitives", choices=["primitives", "terrain"],
                    help="primitives: the primitive-union shell (configs 1, 3, 4); terrain: solid fBm terrain (config 0, 256^3)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--sample-resolution", type=int, default=0, help="CPU sample sub-volume side (0: 256, or the grid)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="skip the CUDA-graph replay of the build (tdag_batch_graph_*)")
    ap.add_argument("--cpu-baseline", default="auto", choices=["auto", "full", "sample"],
                    help="full: the oracle on the whole grid once (auto: up to 2048^3); sample: random sub-volumes only")
    ap.add_argument("--cpu-baseline-timeout", type=float, default=900.0, help="seconds allowed to the whole-grid oracle build")
    ap.add_argument("--workload", default="single", choices=["single", "batch96", "proposal"],
                    help="single: one 2048^3 grid (headline); batch96: 96 grids of 128^3..1024^3 in one batched build; "
                         "proposal: learned source proposals (approximate) against the exhaustive build of the same grid")
    ap.add_argument("--encoder", default="hierarchical", choices=["hierarchical", "block"],
                    help="proposal: children in canonical octant order with an MLP per level (the configured encoder), or the "
                         "mean-pooled block MLP")
    ap.add_argument("--train-grids", type=int, default=20, help="proposal: seeded 1024^3 training grids")
    ap.add_argument("--train-steps", type=int, default=10000,
                    help="proposal: training steps of 2048 positive pairs each (10000: 2.05e7 positive pairs)")
    ap.add_argument("--grids", type=int, default=96)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--probe-bulk-copy", type=int, default=0, choices=[0, 1, 2],
                    help="level-4 probe source staging: 1 = bulk copy (TMA) one source ahead, 0/2 = cooperative loads")
    return ap.parse_args()


def batch_specs(count: int, seed: int):
    """96 seeded scenes: sides log-uniform in 128..1024 (powers of two), 0.1%..5% shell voxels.
    Shell voxels grow like primitives x side^2 with this generator (4000 primitives at 2048^3 give
    ~1.2% shell voxels), so the primitive count for density d at side r is 4000 (d / 0.012) (r / 2048)."""
    import tdag
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        side = 1 << int(round(rng.uniform(7, 10)))
        density = rng.uniform(0.001, 0.05)
        prims = max(4, int(round(4000 * (density / 0.012) * (side / 2048))))
        specs.append(tdag.SceneSpec(kind=tdag.SCENE_PRIMITIVES, resolution=side, seed=seed * 1000 + i, num_primitives=prims))
    return specs


def run_proposal(args, world, rank, local, pg):
    """Learned source proposals (approximate mode): train the encoder on exhaustive labels of seeded
    1024^3 grids, then build the bench grid exhaustively and with k = 8 and 32 proposals per target.
    Reports build time, total nodes and extra nodes against the exhaustive build; every proposed
    match is verified exactly, so every result is a valid TDAG."""
    import torch
    import tdag
    from tdag import proposal as P

    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    ctx = tdag.Context(dev)
    cfg = tdag.TransformDAGConfig()
    t0 = time.perf_counter()
    sets = []
    for seed in range(100, 100 + args.train_grids):
        spec = tdag.SceneSpec(kind=tdag.SCENE_PRIMITIVES, resolution=1024, seed=seed, num_primitives=args.primitives // 2)
        g = tdag.scene_svdag(spec, to_dag=True, ctx=ctx)
        for level, words in P.level_items(g, cfg, ctx=ctx).items():
            sets.append((words, level, P.exhaustive_parents(ctx, words, level, cfg)[0]))
        g.free()
    t_labels = time.perf_counter() - t0
    enc = (P.HierarchicalEncoder if args.encoder == "hierarchical" else P.ProposalEncoder)(seed=0, ctx=ctx)
    t0 = time.perf_counter()
    losses = P.train(enc, sets, steps=args.train_steps, batch=2048)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del sets
    spec = scene_spec(args)
    g = tdag.scene_svdag(spec, to_dag=True, ctx=ctx)
    voxels = g.voxel_count

    def nodes_of(r):
        h = r.to_host(ctx=ctx)
        n = int(sum(len(a) for a in h.nodes_per_level) + len(h.sub_grids))
        r.free()
        return n

    def timed(fn):
        for _ in range(max(args.warmup, 1)):
            out = fn()
            out[0].free() if isinstance(out, tuple) else out.free()
        best = None
        for _ in range(max(args.steps, 1)):
            torch.cuda.synchronize()
            t = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            best = dt if best is None or dt < best else best
            keep = out
        return best, keep

    ex_s, ex = timed(lambda: tdag.construct_transform_dag_device(g, cfg, ctx=ctx))
    ex_nodes = nodes_of(ex)
    # the ceiling of any proposal method: only the exhaustive result's parents search (no network)
    parents = P.exhaustive_parent_sets(g, cfg, ctx=ctx)
    best_s, (best, best_src) = timed(lambda: P.construct_transform_dag_with_sources(g, parents, cfg, ctx=ctx))
    best_nodes = nodes_of(best)
    # recall@8 of the exhaustive parents: learned lists against the no-network lists
    recall = {}
    for level, words in P.level_items(g, cfg, ctx=ctx).items():
        parent, _ = P.exhaustive_parents(ctx, words, level, cfg)
        pos = P.popcount_positions(words)
        recall[str(level)] = {"learned": P.recall_at_k(P.propose_lists(P.embed(enc, words, level), pos, 8, ctx), parent),
                              "popcount_neighbours": P.recall_at_k(P.popcount_neighbour_lists(pos, 8), parent),
                              "random": P.recall_at_k(P.random_lists(pos, 8), parent)}
    # no-network selectors: a fraction of the items searches (the first in the source order, or random)
    fractions = []
    for rule in ("popcount", "random"):
        for rho in (0.2, 0.5, 0.7):
            s_f, (r, src) = timed(lambda: P.construct_transform_dag_by_fraction(g, rule, rho, cfg, ctx=ctx))
            n_f = nodes_of(r)
            fractions.append({"rule": rule, "fraction": rho, "ms": s_f * 1e3, "speed_vs_exhaustive": ex_s / s_f,
                              "extra_nodes_percent": 100.0 * (n_f - ex_nodes) / ex_nodes})
    modes = {}
    for k in (8, 32):
        s_k, (r, src) = timed(lambda: P.construct_transform_dag_proposed(g, enc, k, cfg, ctx=ctx))
        n_k = nodes_of(r)
        secs = getattr(P.construct_transform_dag_proposed, "last_seconds", {})
        modes[str(k)] = {"ms": s_k * 1e3, "mvoxels_per_s": voxels / s_k / 1e6, "nodes": n_k,
                         "extra_nodes_percent": 100.0 * (n_k - ex_nodes) / ex_nodes, "speed_vs_exhaustive": ex_s / s_k,
                         "embed_ms_per_level": {str(l): v[0] * 1e3 for l, v in secs.items()},
                         "score_ms_per_level": {str(l): v[1] * 1e3 for l, v in secs.items()},
                         "sources_per_level": {str(l): {"items": it, "sources": sc} for l, (it, sc) in src.items()}}
    out = {"metric": "TDAG build Mvoxels/s (learned proposals, approximate)", "value": modes["8"]["mvoxels_per_s"], "unit": UNIT,
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "u64 (encoder bf16)",
           "data": "synthetic (device-generated primitive scenes; training grids seeded 100..)", "config": workload_config(args, voxels),
           "exhaustive": {"ms": ex_s * 1e3, "mvoxels_per_s": voxels / ex_s / 1e6, "nodes": ex_nodes},
           "parents_only": {"ms": best_s * 1e3, "speed_vs_exhaustive": ex_s / best_s, "nodes": best_nodes,
                            "sources_per_level": {str(l): {"items": it, "sources": sc} for l, (it, sc) in best_src.items()},
                            "note": "only the exhaustive result's parents search, no network: the ceiling of any proposal method"},
           "proposal": modes,
           "fraction_baselines": fractions,
           "recall_at_8": recall,
           "training": {"encoder": args.encoder, "grids": args.train_grids, "resolution": 1024, "steps": args.train_steps, "label_s": t_labels, "train_s": t_train,
                        "positive_pairs_max": args.train_steps * 2048, "in_batch_negative_pairs_max": args.train_steps * 2048 * 2047,
                        "loss_first": losses[0] if losses else None, "loss_last": losses[-1] if losses else None}}
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_batch(args, world, rank, local, pg):
    """Config 2: independent grids of uneven size through one batched build (tdag_build_batched_device),
    autotuned; every grid's result is checked against its own single-grid build."""
    import torch
    import tdag
    from tdag import autotune

    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    ctx = tdag.Context(dev)
    # the batch's grids are independent: rank r builds grids r, r + N, ... of the same seeded set
    all_specs = batch_specs(args.grids, args.seed)
    specs = all_specs[rank::world]
    devs = [tdag.scene_svdag(sp, to_dag=True, ctx=ctx) for sp in specs]
    voxels = sum(d.voxel_count for d in devs)
    if pg is not None:
        import torch as _t
        tv = _t.tensor([float(voxels)], dtype=_t.float64, device=f"cuda:{dev}")
        pg.all_reduce(tv)
        total_voxels = int(tv.item())
    else:
        total_voxels = voxels
    cfg = tdag.TransformDAGConfig()
    tuning, tune_ms, table = ({}, None, [])
    if not args.no_autotune:
        tuning, tune_ms, table = autotune.autotune_batched(devs, cfg, device=dev, repeats=2)
    tctx = tdag.Context(dev, tuning)
    for _ in range(max(args.warmup, 0)):
        res, _ = tdag.construct_transform_dag_batched_device(devs, cfg, ctx=tctx)
        for r in res:
            r.free()
    clocks = ClockSampler(dev)
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    dev_ms, launches, last = 0.0, 0, None
    for _ in range(args.steps):
        res, st = tdag.construct_transform_dag_batched_device(devs, cfg, ctx=tctx)
        dev_ms += st["total_ms"]
        launches += st["kernel_launches"]
        if last is not None:  # keep only the last step's results for the exactness check
            for r in last:
                r.free()
        last = res
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop()
    # exactness against per-grid builds, and the per-grid device time for comparison
    per_grid_ms = 0.0
    exact = True
    for d, r in zip(devs, last):
        single = tdag.construct_transform_dag_device(d, cfg, ctx=tctx)
        per_grid_ms += single.stats["total_ms"]
        exact &= single.to_host(tctx).to_bytes() == r.to_host(tctx).to_bytes()
        single.free()
        r.free()
    # the same build captured in one CUDA graph (tdag_batch_graph_*), against the eager call, both
    # timed around the whole call (host round trips and result copies included)
    graph_info = None
    if not args.no_graph:
        def call_ms(fn, reps):
            ms = []
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                res, st = fn()
                torch.cuda.synchronize()
                ms.append((time.perf_counter() - t0) * 1e3)
                for r in res:
                    r.free()
            return float(statistics.median(ms)), st
        eager_call, _ = call_ms(lambda: tdag.construct_transform_dag_batched_device(devs, cfg, ctx=tctx), max(args.steps, 3))
        t0 = time.perf_counter()
        graph = tdag.BatchGraph(devs, cfg, ctx=tctx)
        create_ms = (time.perf_counter() - t0) * 1e3
        first, _ = graph.launch()
        g_exact = True
        for d, r in zip(devs, first):
            single = tdag.construct_transform_dag_device(d, cfg, ctx=tctx)
            g_exact &= single.to_host(tctx).to_bytes() == r.to_host(tctx).to_bytes()
            single.free()
            r.free()
        graph_call, gst = call_ms(graph.launch, max(args.steps, 3))
        graph.free()
        graph_info = {"call_ms": graph_call, "device_ms": gst["total_ms"], "kernel_nodes": gst["kernel_launches"], "create_ms": create_ms,
                      "eager_call_ms": eager_call, "speedup_vs_eager_call": eager_call / graph_call if graph_call > 0 else None,
                      "bit_exact_vs_per_grid": bool(g_exact)}
    dev_ms = max_over_ranks(pg, dev_ms)
    value = total_voxels * args.steps / (dev_ms / 1e3) / 1e6  # the whole batch over the slowest rank's time
    out = {
        "metric": "TDAG batched build Mvoxels/s", "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (device-generated primitive scenes)",
        "config": {"workload": f"{len(all_specs)} independent grids, sides log-uniform 128..1024, 0.1-5% shell voxels, one batched build "
                               f"per GPU over its share of the grids (grid i on rank i mod {world})",
                   "sides": sorted(sp.resolution for sp in all_specs), "solid_voxels": int(total_voxels),
                   "l2": "inputs resident; no flush (each step re-reads the whole batch)"},
        "autotune": {"chosen": tuning, "candidates": [{"tuning": t, "ms": m} for t, m in table]},
        "bit_exact_vs_per_grid": bool(exact),
        "per_grid_sum_ms": per_grid_ms,
        "speedup_vs_per_grid": per_grid_ms / (dev_ms / args.steps) if dev_ms > 0 else None,
        "clocks": clk, "gpu_launches": int(launches),
    }
    if graph_info is not None:
        out["graph"] = graph_info
    if rank == 0:
        print(json.dumps(out), flush=True)


def scene_spec(args):
    import tdag
    if getattr(args, "scene", "primitives") == "terrain":
        return tdag.SceneSpec(kind=tdag.SCENE_TERRAIN, resolution=args.resolution, seed=args.seed, shell=False)
    return tdag.SceneSpec(kind=tdag.SCENE_PRIMITIVES, resolution=args.resolution, seed=args.seed, num_primitives=args.primitives)


def cpu_samples(args, count: int, side: int = 0, seed: int = 12345):
    """`count` aligned side^3 sub-volumes of the workload's grid, drawn without replacement (seeded)
    among the non-empty ones and reused cyclically when there are fewer, as (.svo bytes of the SVDAG,
    solid voxels, origin). Generated on the CPU by the oracle's scene statement: the restriction of
    the whole grid to each sub-box, shell included (scene_oracle.cpp). The config-0 terrain is small
    enough to be its own sample."""
    from oracle import generator
    from oracle import oracle as orc
    orc.build()
    if getattr(args, "scene", "primitives") == "terrain":
        dense = generator.terrain(args.resolution, args.seed)
        svo = orc.to_dag(orc.svo_from_dense(dense))
        return [(svo, int(dense.sum()), (0, 0, 0))] * count
    side = min(side or args.sample_resolution or 256, args.resolution)
    per = args.resolution // side
    rng = np.random.default_rng(seed)
    out = []
    for idx in rng.permutation(per ** 3):
        if len(out) == count:
            break
        origin = (int(idx % per) * side, int(idx // per % per) * side, int(idx // (per * per)) * side)
        dense = orc.scene_dense(args.resolution, args.seed, args.primitives, origin=origin, size=side)
        vox = int(dense.sum())
        if vox:
            out.append((orc.to_dag(orc.svo_from_dense(dense)), vox, origin))
    return [out[i % len(out)] for i in range(count)] if out else []


def oracle_build_seconds(svo: bytes) -> float:
    """One oracle constructTransformDAG (default config) on .svo bytes, all host threads: seconds."""
    from oracle import oracle as orc
    orc.build()
    t0 = time.perf_counter()
    orc.construct_tdag(svo, True, True, True, 4)
    return time.perf_counter() - t0


def _oracle_child(svo: bytes, q):
    q.put(oracle_build_seconds(svo))


def oracle_build_seconds_limited(svo: bytes, timeout_s: float):
    """oracle_build_seconds in a spawned child process, given up after timeout_s (None then)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_oracle_child, args=(svo, q), daemon=True)
    p.start()
    try:
        return q.get(timeout=timeout_s)
    except Exception:
        return None
    finally:
        if p.is_alive():
            p.terminate()
        p.join(timeout=10)


def workload_config(args, voxels=None):
    if getattr(args, "scene", "primitives") == "terrain":
        what = f"{args.resolution}^3 solid fBm terrain (5 octaves, base frequency 1/64, seed {args.seed})"
    else:
        what = (f"{args.resolution}^3 primitive-union shell ({args.primitives} primitives, 30% transformed copies, "
                f"seed {args.seed})")
    cfg = {
        "workload": f"single-grid exhaustive TDAG build, {what}, symmetry+axis permutation+translation, maxTranslationLevel 4",
        "resolution": args.resolution,
        "scene": getattr(args, "scene", "primitives"),
        "primitives": args.primitives if getattr(args, "scene", "primitives") == "primitives" else 0,
        "seed": args.seed,
        "l2": "flushed between timed steps (256 MiB device write)",
    }
    if voxels is not None:
        cfg["solid_voxels"] = int(voxels)
    return cfg


# ------------------------------------------------------------------------------------------------
# distributed helpers (torchrun: one process per GPU, replicas)
# ------------------------------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def replica_value(voxels_per_rank: int, steps: int, world: int, max_seconds: float) -> float:
    """Whole-job Mvoxels/s of N replicas: every rank builds the same workload, so the job's voxels
    are world x steps x voxels, over the slowest rank's time."""
    return voxels_per_rank * steps * world / max_seconds / 1e6


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
# roofline of the dominant kernel
# ------------------------------------------------------------------------------------------------
GRID_BYTES = {2: 8, 3: 64, 4: 512}


def search_model_bytes(level: int, st: dict) -> float:
    """The probe kernel's algorithmic bytes in the cost model of the search (one R^3 grid read per
    source item, one 16-byte (hash, range) slot per non-empty probe): M*G + P*16."""
    return st["items"] * GRID_BYTES[level] + st["probes"] * 16


def build_model_bytes(st_all: dict) -> float:
    """Algorithmic bytes of a whole build in the same cost model: the hierarchical pass (read node, gather
    8 child pointers, write mapping, write unique) plus, per translation level, items (grid, 8 corner
    entries, parent), 16 bytes per probe, two grids per verification and the resolve pass."""
    b = 0.0
    for lvl, h in st_all["hierarchical"].items():
        n, u = h["items"], h["unique"]
        b += n * (8 + 16) + u * 8 if int(lvl) == 2 else n * (32 + 8 * 16 + 16) + u * 64
    for lvl, t in st_all["translation"].items():
        G = GRID_BYTES[int(lvl)]
        m = t["items"]
        b += m * (G + 8 * 16 + 8) + t["probes"] * 16 + t["verifications"] * 2 * G + m * 8
    return b


def probe_algorithmic_bytes(level: int, st: dict) -> float:
    """Probe kernel of one level (DRAM): every source grid read once (M*G), its three line
    orientations written for verification (M*3R^2*2), one 16-byte record per filter survivor (F*16).
    The filter words the probes read (4 bytes each) stay in L2 and are counted in l2_probe instead."""
    R = 1 << level
    G = GRID_BYTES[level]
    return st["items"] * G + st["items"] * 3 * R * R * 2 + st["filter_pass"] * 16


def l2_probe_peak(ctx) -> float:
    """Random 4-byte loads per second from an L2-resident buffer: the maximum over 4, 16 and 64 MiB."""
    import tdag
    from tdag import _abi
    best = 0.0
    for mib in (4, 16, 64):
        v = ctypes.c_double(0.0)
        _abi.check(tdag.lib().tdag_l2_probe_peak(ctx.handle, mib << 20, 1 << 30, ctypes.byref(v)))
        best = max(best, v.value)
    return best


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(level: int, args):
    """DRAM bytes (read + write) of the level's probe launches in one build of this workload, from an
    ncu capture of the same workload if one is recorded (else None)."""
    p = os.path.join(REPO, "profiles", "probe_traffic.json")
    if not os.path.exists(p):
        return None
    key = f"{getattr(args, 'scene', 'primitives')}/{args.resolution}/{args.primitives}/{args.seed}"
    try:
        with open(p) as f:
            d = json.load(f)
        return d.get("workloads", {}).get(key, {}).get(str(level))
    except (OSError, ValueError, AttributeError):
        return None


# ------------------------------------------------------------------------------------------------
def run_reference(args, world, rank, pg):
    """Reference arm: the CPU restatement of the reference path (pinned byte for byte to the reference's
    own code; all host threads), one seeded random aligned sub-volume of the same grid per step,
    generated on the CPU. Loads no product library. Only rank 0 works."""
    if rank != 0:
        barrier(pg)
        return
    from oracle import oracle as orc
    orc.build()
    cores = orc.max_threads()
    samples = cpu_samples(args, max(args.warmup, 0) + args.steps)
    for svo, _, _ in samples[: max(args.warmup, 0)]:
        oracle_build_seconds(svo)
    times, voxels = [], 0
    for svo, vox, _ in samples[max(args.warmup, 0):]:
        times.append(oracle_build_seconds(svo))
        voxels += vox
    total = sum(times)
    value = voxels / total / 1e6
    side = min(args.sample_resolution or 256, args.resolution)
    what = ("the whole 256^3 terrain per step" if getattr(args, "scene", "primitives") == "terrain" else
            f"a different seeded random aligned {side}^3 sub-volume of the same grid per step ({voxels} solid voxels over "
            f"{args.steps} steps), generated on the CPU")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / len(times) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic", "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": what},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(pg)


def run_ours(args, world, rank, local, pg):
    import torch
    import tdag
    from tdag import _abi

    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    ctx = tdag.Context(dev, {"probe_bulk_copy": args.probe_bulk_copy})
    spec = scene_spec(args)
    g = tdag.scene_svdag(spec, to_dag=True, ctx=ctx)
    voxels = g.voxel_count
    cfg = tdag.TransformDAGConfig()
    sp = ctypes.c_void_p()
    _abi.check(tdag.lib().tdag_ctx_stream(ctx.handle, ctypes.byref(sp)))
    lib_stream = torch.cuda.ExternalStream(sp.value, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    def step():
        r = tdag.construct_transform_dag_device(g, cfg, ctx=ctx)
        st = r.stats
        r.free()
        return st

    for _ in range(max(args.warmup, 0)):
        step()
    # ---- timed, device-resident
    clocks = ClockSampler(dev)
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    dev_ms, stats_list = 0.0, []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        st = step()
        e1.record(lib_stream)
        e1.synchronize()
        dev_ms += e0.elapsed_time(e1)
        stats_list.append(st)
        print(f"[bench] step {len(stats_list)}: {e0.elapsed_time(e1):.2f} ms (library {st['total_ms']:.2f} ms)", file=sys.stderr, flush=True)
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop()
    dev_ms = max_over_ranks(pg, dev_ms)
    value = replica_value(voxels, args.steps, world, dev_ms / 1e3)

    # ---- the same build replayed from one CUDA graph (tdag_batch_graph_*, a batch of one grid), timed
    # the same way around the whole call: the input check, the graph and the result copies
    graph_info = None
    if not args.no_graph:
        t0 = time.perf_counter()
        bg = tdag.BatchGraph([g], cfg, ctx=ctx)
        create_ms = (time.perf_counter() - t0) * 1e3
        first, _ = bg.launch()
        ref = tdag.construct_transform_dag_device(g, cfg, ctx=ctx)
        g_exact = first[0].to_host(ctx).to_bytes() == ref.to_host(ctx).to_bytes()
        ref.free()
        first[0].free()
        gms, gdev = [], []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(lib_stream)
            res, gst = bg.launch()
            e1.record(lib_stream)
            e1.synchronize()
            gms.append(e0.elapsed_time(e1))
            gdev.append(gst["total_ms"])
            for r in res:
                r.free()
        bg.free()
        gms_mean = max_over_ranks(pg, sum(gms)) / args.steps
        graph_info = {"ms_per_step": gms_mean, "value": replica_value(voxels, args.steps, world, gms_mean * args.steps / 1e3),
                      "graph_device_ms": sum(gdev) / len(gdev), "kernel_nodes": gst["kernel_launches"], "create_ms": create_ms,
                      "bit_exact_vs_eager": bool(g_exact),
                      "note": "tdag_batch_graph_launch per step: device check of the input against the graph's snapshot, one cudaGraphLaunch, result copies"}

    # ---- e2e through tdag_build with pinned host buffers
    host = g.to_host()
    keep = []
    view = _abi.SvdagView()
    view.resolution, view.root_level, view.structure_type = host.resolution, host.root_level, host.structure_type
    h2d = 0
    for lvl in range(3, host.root_level + 1):
        a = host.nodes_per_level[lvl]
        pt = torch.empty(a.size, dtype=torch.int32, pin_memory=True)
        pn = pt.numpy().view(np.uint32)
        pn[:] = a.reshape(-1)
        keep.append(pt)
        view.nodes[lvl] = ctypes.cast(pn.ctypes.data, ctypes.POINTER(ctypes.c_uint32))
        view.node_counts[lvl] = a.shape[0]
        h2d += a.nbytes
    lt = torch.empty(host.sub_grids.size, dtype=torch.int64, pin_memory=True)
    ln = lt.numpy().view(np.uint64)
    ln[:] = host.sub_grids
    keep.append(lt)
    view.leaves = ctypes.cast(ln.ctypes.data, ctypes.POINTER(ctypes.c_uint64))
    view.leaf_count = host.sub_grids.size
    h2d += host.sub_grids.nbytes
    cfg_c = tdag._config_struct(cfg)
    d2h = 0
    e2e_s = 0.0
    e2e_steps = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        rp = ctypes.POINTER(_abi.Result)()
        t0 = time.perf_counter()
        _abi.check(tdag.lib().tdag_build(ctx.handle, ctypes.byref(view), ctypes.byref(cfg_c), ctypes.byref(rp)))
        dt = time.perf_counter() - t0
        r = rp.contents
        d2h = sum(r.node_counts[l] * 64 for l in range(3, r.root_level + 1)) + r.leaf_count * 8
        tdag.lib().tdag_result_free(rp)
        if i >= args.warmup:
            e2e_s += dt
            e2e_steps.append(dt * 1e3)
    e2e_s = max_over_ranks(pg, e2e_s)
    e2e_value = replica_value(voxels, args.steps, world, e2e_s)

    # ---- the rest of the pipeline, outside the timed region: SVO + toDAG of the scene on the device,
    # the .tdag16 encoding of the result (pointer tables + Huffman, the renderer's format; the file
    # bytes copied to the host) and the lossless check of the file against the source SVDAG
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g2 = tdag.scene_svdag(spec, to_dag=True, ctx=ctx)
    torch.cuda.synchronize()
    svdag_ms = (time.perf_counter() - t0) * 1e3
    g2.free()
    enc_cfg = tdag.TransformEncodingConfig(pointer_tables=True, huffman_code=True)
    r = tdag.construct_transform_dag_device(g, cfg, ctx=ctx)
    enc_ms, enc_wall = [], []
    for i in range(max(args.warmup, 1) + args.steps):
        data, est = tdag.construct_transform_dag16(r, cfg, enc_cfg, ctx=ctx, return_stats=True)
        if i >= max(args.warmup, 1):
            enc_ms.append(est["encode_ms"])
            enc_wall.append(est["wall_ms"])
    r.free()
    d16 = tdag.Tdag16Device(data, ctx=ctx)
    d16.verify(g)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ver = d16.verify(g)
    torch.cuda.synchronize()
    verify_ms = (time.perf_counter() - t0) * 1e3
    d16.free()
    build_ms = dev_ms / args.steps
    encode_wall_ms = sum(enc_wall) / len(enc_wall)
    pipeline = {
        "svdag_ms": svdag_ms, "build_ms": build_ms, "encode16_ms": encode_wall_ms,
        "total_ms": svdag_ms + build_ms + encode_wall_ms,
        "mvoxels_per_s": voxels / ((svdag_ms + build_ms + encode_wall_ms) / 1e3) / 1e6,
        "note": "scene generation + SVO + toDAG on the device, the build, and the .tdag16 encoding with the file copied to the host",
    }
    tdag16 = {"bytes": len(data), "encoding": "pointer tables + Huffman", "encode_device_ms": sum(enc_ms) / len(enc_ms),
              "encode_wall_ms": encode_wall_ms, "kernel_launches": est["kernel_launches"], "verify_ms": verify_ms,
              "lossless": ver["existence_mismatches"] == 0 and ver["voxel_mismatches"] == 0,
              "verify": {k: ver[k] for k in ("existence_mismatches", "voxel_mismatches", "boxes_compared", "box_level")}}

    # ---- roofline of the dominant kernel: the probe kernel of the level with the largest probe time
    last = stats_list[-1]
    lvl_times = {L: sum(s["translation"][L]["search_ms"] for s in stats_list) / len(stats_list) for L in (2, 3, 4)}
    probe_times = {L: sum(s["translation"][L]["probe_ms"] for s in stats_list) / len(stats_list) for L in (2, 3, 4)}
    dom = max(probe_times, key=lambda L: probe_times[L])
    ms = probe_times[dom]
    st = last["translation"][dom]
    alg = search_model_bytes(dom, st)
    achieved = alg / (ms / 1e3) / 1e9 if ms > 0 else None
    peak, peak_kind = load_peaks()
    dram_alg = probe_algorithmic_bytes(dom, st)
    l2_peak = l2_probe_peak(ctx)
    probes_per_s = st["probes"] / (ms / 1e3) if ms > 0 else None
    build_bytes = build_model_bytes(last)
    build_s = dev_ms / args.steps / 1e3
    roof = {"bound": "l2", "kernel": f"probeKernel<R={1 << dom}> (translation level {dom})", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
            "traffic": load_traffic(dom, args), "algorithmic_bytes": alg, "device_ms": ms,
            "model": "algorithmic bytes of the search's cost model: M*G + P*16 (M source items, G grid bytes, P non-empty probes)",
            "dram_only": {"algorithmic_bytes": dram_alg, "achieved": dram_alg / (ms / 1e3) / 1e9 if ms > 0 else None,
                          "note": "grids in + line orientations and survivor records out; the filter stays in L2"},
            "l2_probe": {"achieved_loads_per_s": probes_per_s, "peak_loads_per_s": l2_peak,
                         "frac": (probes_per_s / l2_peak) if probes_per_s and l2_peak else None,
                         "peak_source": "tdag_l2_probe_peak on this GPU (max over 4/16/64 MiB buffers)"},
            "whole_build": {"algorithmic_bytes": build_bytes, "achieved": build_bytes / build_s / 1e9,
                            "frac": build_bytes / build_s / 1e9 / peak}}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic (device-generated primitive scene; no public dataset)",
        "config": workload_config(args, voxels),
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step_ms": [round(x, 3) for x in e2e_steps]},
        "clocks": clk,
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats_list)),
        "subgrids_matched_per_s": sum(last["translation"][L]["items"] for L in (2, 3, 4)) / (dev_ms / args.steps / 1e3),
        # the reference's own search throughput figure (find_translation.cpp:879-885): sources x R^3 voxels
        # x 8 fold directions x 6 axis permutations x 8-byte hashes per second of search, per level
        "search_permuted_voxel_mib_s": {str(L): (last["translation"][L]["items"] * (1 << (3 * L)) * 8 * 6 * 8 / (lvl_times[L] / 1e3) / 2 ** 20
                                                 if lvl_times[L] > 0 else None) for L in (2, 3, 4)},
        "dense_gvoxels_per_s": {"value": args.resolution ** 3 / (dev_ms / args.steps / 1e3) / 1e9,
                                "note": "resolution^3 cells (empty included) per second of build"},
        "pipeline": pipeline,
        "tdag16": tdag16,
        "stage_ms": {"hierarchical": last["hierarchical_ms"], "translation": last["translation_ms"],
                     "search_L4": lvl_times[4], "search_L3": lvl_times[3], "search_L2": lvl_times[2],
                     "probe_L4": probe_times[4], "probe_L3": probe_times[3], "probe_L2": probe_times[2]},
    }
    if graph_info is not None:
        out["graph"] = graph_info
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as orc
        orc.build()
        cores = orc.max_threads()
        samples = cpu_samples(args, 8)
        sdt = sum(oracle_build_seconds(svo) for svo, _, _ in samples)
        svox = sum(v for _, v, _ in samples)
        side = min(args.sample_resolution or 256, args.resolution)
        sample = {"value": svox / sdt / 1e6, "unit": UNIT, "cores": cores,
                  "sample": f"8 seeded random aligned {side}^3 sub-volumes of the same grid ({svox} solid voxels), {sdt:.1f} s"}
        mode = args.cpu_baseline if args.cpu_baseline != "auto" else ("full" if args.resolution <= 2048 else "sample")
        full_s = oracle_build_seconds_limited(host.to_svo_bytes(), args.cpu_baseline_timeout) if mode == "full" else None
        if full_s:
            out["cpu_baseline"] = {"value": voxels / full_s / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
                                   "sample": f"the whole grid ({voxels} solid voxels): one oracle build of its SVDAG, {full_s:.1f} s",
                                   "sample_subvolumes": sample}
        else:
            why = "" if mode == "sample" else f" (the whole-grid build did not finish within {args.cpu_baseline_timeout:.0f} s)"
            out["cpu_baseline"] = dict(sample, kind="port", sample=sample["sample"] + why)
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    elif args.workload == "batch96":
        run_batch(args, world, rank, local, pg)
    elif args.workload == "proposal":
        run_proposal(args, world, rank, local, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
