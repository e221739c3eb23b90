"""The multi-replica path of bench.py on CPU: two ranks over gloo (one process each),
the timing barrier, the max over ranks, and the reference arm run by rank 0 alone. The
path has no data-path collective: replicas solve their own planets."""
import contextlib
import io
import json
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, local = bench.dist_env()
    dist = bench.init_dist(w, "gloo")
    bench.barrier(dist)
    slowest = bench.max_over_ranks(0.5 + r, dist)    # rank r "took" 0.5 + r seconds
    bench.barrier(dist)

    class Args:
        workload, seed, steps, warmup = "batch", 1, 1, 1

    printed = io.StringIO()
    with contextlib.redirect_stdout(printed):
        bench.run_reference(Args, r, w)
    out.put((r, w, local, slowest, printed.getvalue()))
    dist.destroy_process_group()


def test_two_gloo_ranks_time_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    results = sorted(out.get(timeout=5) for _ in procs)
    assert [r[:3] for r in results] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[3] == 1.5 for r in results)          # value uses the slowest rank's time
    assert results[1][4] == ""                        # the reference arm: rank 1 does no work
    line = json.loads(results[0][4])                  # rank 0 prints the one line of the contract
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["value"] == line["value"] == line["e2e"]["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["planets"] == 64 and line["config"]["cells"] == 2252928
