"""Multi-process path of bench.py on CPU: two gloo ranks run replica_throughput (replicas only, no data-path
collective); the job's step time is the slowest rank's and the throughput counts both ranks' work."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    step = 10.0 + 5.0 * rank   # rank 1 is the slow one
    e2e = 20.0 + 1.0 * rank
    q.put((rank, bench.replica_throughput(step, e2e, 1_000_000, world, device="cpu")))
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        step_ms, e2e_ms, value, e2e = out[r]
        assert step_ms == 15.0 and e2e_ms == 21.0
        assert abs(value - 2 * 1e6 / 15e-3 / 1e6) < 1e-9
        assert abs(e2e - 2 * 1e6 / 21e-3 / 1e6) < 1e-9


def test_replica_throughput_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(4.0, 8.0, 4_000_000, 1, device="cpu") == (4.0, 8.0, 1000.0, 500.0)
