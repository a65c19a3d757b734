"""Replica runs across ranks (CPU, gloo, world size 2).

``bench.py --gpus N`` runs one independent structure function per GPU: the
ranks meet at barriers around the timed region, the job time is the slowest
rank's, and the throughput counts every rank's frames.  These are the only
collectives, and ``fastddm_gb300.replicas`` runs them over any process-group
backend, so the multi-rank logic is tested here on CPU processes.
"""

import os
import socket
import time

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world_size, port, frames, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world_size), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from fastddm_gb300 import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        ws, r, local = replicas.world()
        replicas.barrier()
        t0 = time.perf_counter()
        time.sleep(times[rank])  # the rank's "timed region"
        replicas.barrier()
        waited = time.perf_counter() - t0
        slowest = replicas.max_over_ranks(times[rank])
        rate = replicas.aggregate_rate(frames, slowest, ws)
        out.put((rank, ws, r, local, waited, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_replicas_two_ranks_gloo():
    world_size, frames, times = 2, 4000, [0.05, 0.20]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world_size, port, frames, times, out)) for r in range(world_size)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in range(world_size))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ws, r, local, waited, slowest, rate in results:
        assert (ws, r, local) == (world_size, rank, rank)
        # the closing barrier holds every rank until the slowest is done
        assert waited >= max(times) - 1e-3
        # every rank reports the slowest rank's time and the whole job's frames
        assert slowest == max(times)
        assert rate == pytest.approx(world_size * frames / max(times))


def test_single_process_needs_no_group(monkeypatch):
    from fastddm_gb300 import replicas

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.world() == (1, 0, 0)
    replicas.barrier()
    assert replicas.max_over_ranks(1.5) == 1.5
    assert replicas.aggregate_rate(4000, 0.2, 1) == pytest.approx(20000.0)
    with pytest.raises(ValueError):
        replicas.aggregate_rate(10, 0.0, 1)
