"""The multi-GPU path is independent replicas; its only cross-rank step is
the timing of a run (barrier, slowest rank, whole-job throughput). Checked
with two gloo ranks on the host."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    from qubatron_gb300 import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        replicas.barrier()
        # rank r renders 100 * (r + 1) units in 1 + r seconds
        rate, slowest = replicas.job_throughput(100.0 * (rank + 1), 1.0 + rank)
        q.put((rank, replicas.world_size(), rate, slowest, replicas.max_over_ranks(rank * 7.0)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_job_throughput():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, world, rate, slowest, mx in got:
        assert world == 2
        assert slowest == pytest.approx(2.0)       # the slower rank's time
        assert rate == pytest.approx(300.0 / 2.0)  # all ranks' units over it
        assert mx == pytest.approx(7.0)


def test_single_process_is_identity():
    from qubatron_gb300 import replicas
    assert replicas.world_size() == 1
    assert replicas.job_throughput(50.0, 2.0) == (25.0, 2.0)
    replicas.barrier()
