"""Host-side replica bookkeeping of multi-GPU benchmark runs, exercised with
two gloo ranks on CPU (the path has no device-side exchange)."""

from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from titsolver_gb300.replicas import aggregate, init_from_env

    ranks = init_from_env("gloo")
    try:
        ranks.barrier()
        # Rank r processed (r + 1) * 1000 units in (r + 1) seconds.
        value, t_max = aggregate((rank + 1) * 1000.0, float(rank + 1), ranks)
        q.put((rank, value, t_max, ranks.world_size))
    finally:
        ranks.close()


def test_two_rank_aggregate_sums_units_over_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, t_max, world in res:
        assert world == 2
        assert t_max == 2.0
        assert value == pytest.approx(3000.0 / 2.0)


def test_single_rank_needs_no_process_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    from titsolver_gb300.replicas import aggregate, init_from_env

    ranks = init_from_env()
    assert ranks.world_size == 1 and ranks.dist is None
    assert aggregate(10.0, 2.0, ranks) == (5.0, 2.0)
