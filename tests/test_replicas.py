"""The N-rank form of the benchmark on CPU: every rank runs an independent replica of the workload (the coupling on
one mesh per GPU has no exchange step), the job's time is the slowest rank's and its work the sum over ranks.
Two gloo ranks stand in for two GPUs; nothing here launches GPU work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) ms for 1000 * (r + 1) coupling cells
        ms, cells = bench.over_ranks(dist, float(rank + 1), 1000.0 * (rank + 1), "cpu")
        q.put((rank, ms, cells))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_over_ranks_gloo(world):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert [g[0] for g in got] == list(range(world))
    for _, ms, cells in got:
        assert ms == float(world)
        assert cells == 1000.0 * world * (world + 1) / 2


def test_single_rank_is_unchanged():
    import bench
    assert bench.over_ranks(None, 2.5, 1234.0, "cpu") == (2.5, 1234.0)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit without work (the argument object is never read)."""
    import bench
    assert bench.run_reference(None, 1, 2) is None
