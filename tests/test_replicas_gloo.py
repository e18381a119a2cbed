"""Multi-process host logic of bench.py's replica mode, on CPU: two gloo ranks.

The build does not shard (one grid's search is a global join), so N GPUs run N independent replicas:
a barrier around the timed region, the slowest rank's time, and the job's voxels over it. This test
runs that host path with world size 2 over gloo on 127.0.0.1.
"""
import os
import socket
import sys

import pytest

from conftest import REPO


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench

    w, r, local, pg = bench.dist_setup(None)
    try:
        seconds = [1.5, 2.5][rank]  # rank 1 is the slower replica
        bench.barrier(pg)
        slowest = bench.max_over_ranks(pg, seconds)
        value = bench.replica_value(1_000_000, 3, w, slowest)
        bench.barrier(pg)
        out_q.put((r, w, slowest, value))
    finally:
        pg.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    if torch.cuda.is_available():
        pytest.skip("with a GPU, bench.dist_setup picks NCCL and one device per rank")

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort()
    assert [r for r, *_ in results] == [0, 1]
    for _, world, slowest, value in results:
        assert world == 2
        assert slowest == 2.5  # max over ranks
        assert value == pytest.approx(1_000_000 * 3 * 2 / 2.5 / 1e6)  # whole-job voxels over the slowest time


def test_batch_grids_are_partitioned_by_rank():
    """bench.py --workload batch96 on N GPUs: rank r builds grids r, r + N, ... of one seeded set, so
    the shares are disjoint and cover the whole batch (no data-path collective; only the timing and
    the voxel total are reduced)."""
    import sys
    from conftest import REPO
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import bench
    specs = bench.batch_specs(96, 1)
    for world in (1, 2, 4, 8):
        shares = [specs[r::world] for r in range(world)]
        seeds = [sp.seed for sh in shares for sp in sh]
        assert sorted(seeds) == sorted(sp.seed for sp in specs) and len(set(seeds)) == 96
        assert max(len(sh) for sh in shares) - min(len(sh) for sh in shares) <= 1
