"""Replica host logic (bench.py under torchrun) on two gloo ranks on the CPU:
per-rank seeds differ, max-over-ranks picks the slowest rank, and the whole-job
throughput counts every rank's solves over that time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from cunusht_gb300.replicas import Replicas
    R = Replicas(backend="gloo")
    seconds = 1.0 + rank  # rank 1 is the slow replica
    R.barrier()
    out = {"rank": R.rank, "seed": R.seed(1), "max": R.max(seconds), "value": R.throughput(10, seconds)}
    R.barrier()
    R.close()
    q.put(out)


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda r: r["rank"])
    assert res[0]["seed"] != res[1]["seed"]
    assert all(r["max"] == 2.0 for r in res)            # slowest replica
    assert all(abs(r["value"] - 2 * 10 / 2.0) < 1e-12 for r in res)  # 20 solves in 2 s


def test_single_process_is_identity():
    from cunusht_gb300.replicas import Replicas
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    R = Replicas(backend="gloo")
    assert R.world == 1 and R.max(3.5) == 3.5 and R.throughput(4, 2.0) == 2.0
