"""Host logic of bench.py's multi-rank path (one process per GPU under
torchrun), exercised with two gloo ranks on the CPU: per-rank workloads, the
max-over-ranks timing and the whole-job weak-scaling value, and the
reference arm printing on rank 0 only."""
import io
import os
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wall = 1.0 + 0.5 * rank          # rank 1 is the slowest
        wmax = bench.reduce_max(wall)
        value = bench.weak_value(world, 1000, 10, wmax)
        ws, r, local = bench._dist()
        args = type("A", (), {"gpus": world, "steps": 1, "warmup": 3})()
        buf = io.StringIO()
        if rank != 0:
            with redirect_stdout(buf):
                rc = bench.run_reference(args)
        else:
            rc = 0
        q.put((rank, wmax, value, bench.rank_seed(rank), (ws, r, local), rc, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_timing_and_weak_value():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, v0, s0, d0, rc0, out0), (r1, w1, v1, s1, d1, rc1, out1) = res
    assert w0 == w1 == 1.5                     # the slowest rank's time on every rank
    assert v0 == v1 == 2 * 1000 * 10 / 1.5      # whole-job weak-scaling throughput
    assert s0 != s1                             # each rank steps its own columns
    assert d0 == (2, 0, 0) and d1 == (2, 1, 1)
    assert rc1 == 0 and out1 == ""              # the reference arm prints on rank 0 only


def test_fp64_pipe_floor_from_the_committed_profile():
    """bench.py's roofline.fp64_pipe: the committed ncu summary's FP64-pipe
    warp instructions per column-level x 16 cycles over the SMs at the sampled
    clock, and the measured step's fraction of that floor."""
    sys.path.insert(0, str(ROOT))
    import bench
    ipc = bench._profile_figure("fp32", "fp64_warp_inst_per_cl")
    assert ipc is not None and 1.0 < ipc < 200.0
    assert bench._traffic_per_cl("fp32") > 360.0  # measured traffic exceeds the algorithmic bytes
    cl = 345600 * 128
    got = bench.fp64_ceiling("fp32", cl, 25.0, 2070.0, 152)
    floor = ipc * 16 * cl / (152 * 2070e6) * 1e3
    assert got["floor_ms"] == pytest.approx(floor, rel=1e-12)
    assert got["frac"] == pytest.approx(floor / 25.0, rel=1e-12)
    assert bench.fp64_ceiling("fp32", cl, 25.0, None, 152) is None  # no clock sample, no floor
    assert bench.fp64_ceiling("fp64", cl, 400.0, 2070.0, 152)["fp64_warp_inst_per_cl"] > ipc
