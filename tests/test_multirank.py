"""The multi-rank side of bench.py on the CPU: two gloo ranks on 127.0.0.1 (torchrun's
environment variables set by hand). Each rank is an independent replica (the path needs no
collective); the job time is the slowest rank's, the value is world x units / time, and the
reference arm does its work on rank 0 only."""
import os
import queue
import socket
import sys
import time
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")

ROOT = str(Path(__file__).resolve().parents[1])


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.rank_info()
        ms = bench.max_over_ranks([10.0, 25.0, 17.5][rank], w, "cpu")
        out.put(("time", r, w, local, ms, bench.whole_job_rate(1000.0, ms, w)))
        if rank != 0:
            t0 = time.time()
            bench.run_reference(None)  # must return at once, without work or output
            out.put(("ref", r, time.time() - t0))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_ranks_agree_on_the_slowest_time(world):
    ctx = torch.multiprocessing.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = []
    while True:
        try:
            got.append(out.get(timeout=1))
        except queue.Empty:
            break
    times = [g for g in got if g[0] == "time"]
    slowest = max([10.0, 25.0, 17.5][:world])
    assert sorted(g[1] for g in times) == list(range(world))
    assert all(g[2] == world and g[3] == g[1] and g[4] == slowest for g in times)
    assert all(abs(g[5] - world * 1000.0 / slowest / 1e3) < 1e-12 for g in times)
    refs = [g for g in got if g[0] == "ref"]
    assert len(refs) == world - 1 and all(g[2] < 1.0 for g in refs)


def test_single_process_defaults(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.rank_info() == (1, 0, 0)
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.whole_job_rate(8_388_608, 2.5, 1) == pytest.approx(3355.4432)
