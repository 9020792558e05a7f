"""bench.py's multi-rank path on the CPU with two gloo ranks: each rank steps its own replica batch
(different worlds, no exchange), the timing is the slowest rank's, the job rate aggregates all
ranks, and the reference arm runs on rank 0 alone."""
from __future__ import annotations

import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    assert bench.dist_setup() == (ws, rank, rank)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms = bench.reduce_max(10.0 * (rank + 1), dist, "cpu")
        specs = bench.rank_worlds(rank)
        cells = sum(W * H for W, H, *_ in specs)
        cell_sums = [0, 0]
        dist.all_gather_object(cell_sums, cells)
        dist.barrier()
        ref = bench.run_reference(None, ws, rank) if rank != 0 else "skipped"
        out.put((rank, ms, [s[:2] for s in specs[:4]], cell_sums, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, shapes0, cells0, _), (r1, ms1, shapes1, cells1, ref1) = res
    assert ms0 == ms1 == 20.0              # the slowest rank's time on every rank
    assert shapes0 != shapes1              # replicas: each rank its own worlds
    assert cells0 == cells1                # every rank saw both totals
    assert ref1 is None                    # the reference arm: rank 0 alone


class _WallClock:
    def start(self):
        import time
        self.t0 = time.perf_counter()

    def stop(self):
        import time
        self.t1 = time.perf_counter()

    def ms(self):
        return (self.t1 - self.t0) * 1e3


def _replica_rank(rank, ws, port, out):
    """run_engine's replica bookkeeping with the CPU oracle standing in for the engine: each rank
    steps the two smallest worlds of its own batch inside bench.timed_region, the slowest rank's
    time comes back on every rank, and the job rate counts every rank's cells."""
    sys.path.insert(0, str(ROOT))
    import bench
    import oracle as O

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        s = O.baseline_settings()
        specs = sorted(bench.rank_worlds(rank), key=lambda x: x[0] * x[1])[:2]
        worlds = []
        for W, H, P, gs, wsd in specs:
            h, ids, pl = O.generate_world(W, H, P, 1.0, gs)
            worlds.append(O.OracleWorld(s, h, ids, pl, wsd))
        before = [w.h.copy() for w in worlds]

        def step(n):
            for w in worlds:
                w.step(n)

        mine, slowest = bench.timed_region(step, 2, _WallClock(), lambda: None, dist.barrier,
                                           lambda x: bench.reduce_max(x, dist, "cpu"))
        cells = sum(W * H for W, H, *_ in specs)
        moved = all(not (w.h == b).all() for w, b in zip(worlds, before))
        cells_all = bench.reduce_sum(cells, dist, "cpu")
        out.put((rank, mine, slowest, cells, [sp[:2] for sp in specs], moved,
                 bench.job_rate(cells_all, 2, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_step_their_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, mine0, slow0, cells0, shapes0, moved0, rate0), (_, mine1, slow1, cells1, shapes1, moved1, rate1) = res
    assert moved0 and moved1                         # both replicas stepped
    assert shapes0 != shapes1                        # each rank its own worlds
    assert slow0 == slow1 == max(mine0, mine1)       # the slowest rank's time on every rank
    assert cells0 != cells1                          # replicas of different sizes
    assert rate0 == rate1 == pytest.approx((cells0 + cells1) * 2 / (slow0 / 1e3))  # every rank's own cells


def test_job_rate_aggregates_ranks():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.job_rate(1000, 4, 2.0) == pytest.approx(2.0e6)
    assert bench.job_rate(1000 + 3000, 4, 2.0) == pytest.approx(8.0e6)


def test_rooflines_from_the_committed_profiles():
    """The per-cell DRAM traffic and warp-instruction counts bench.py reports come from the committed
    ncu summaries (the marching kernel's traffic captured on the batch, the tile kernel's on a 2048^2
    launch); the issue roofline is achieved / (SMs x 4 x clock)."""
    sys.path.insert(0, str(ROOT))
    import bench

    for v in (bench.MARCH_VARIANT, 4):
        tpc, ipc = bench.profiled_traffic_per_cell(v), bench.profiled_instructions_per_cell(v)
        assert tpc is not None and 40 < tpc < 80      # about 50-71 B/cell against 56 algorithmic
        assert ipc is not None and 5 < ipc < 40       # warp-instructions per cell
    tpc, ipc = bench.profiled_traffic_per_cell(4), bench.profiled_instructions_per_cell(4)
    assert ipc is not None and 5 < ipc < 40           # warp-instructions per cell
    r = bench.issue_roofline(ipc, 2048 * 2048, 0.1, 2070.0, 152)
    assert r["bound"] == "issue" and abs(r["peak"] - 152 * 4 * 2.07) < 1e-9
    assert abs(r["achieved"] - ipc * 2048 * 2048 / 1e-4 / 1e9) < 1e-6
    assert 0 < r["frac"] < 1
    assert bench.issue_roofline(None, 1, 1.0, 2070.0, 152) is None
    assert bench.issue_roofline(ipc, 1, 1.0, None, 152) is None


def test_reference_arm_prints_the_engine_arms_config(capsys):
    """Both arms of bench.py print the same `config` for the headline workload, so the two lines
    compare as one workload; the reference arm's line is complete without a GPU."""
    import json
    import types

    sys.path.insert(0, str(ROOT))
    import bench

    args = types.SimpleNamespace(steps=1, warmup=1, gpus=1)
    bench.run_reference(args, 1, 0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["config"] == bench.workload_config()
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["value"] == line["value"]
