"""The N>1 bench path on CPU ranks (gloo, world size 2): the path has no
exchange step, so N GPUs run independent replicas; the only collective is
the max-over-ranks reduction of the timed region, and the reference arm runs
on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    t = bench.max_over_ranks(1.5 + rank, dist, "cpu")

    class A:
        steps, warmup = 1, 3
    # the reference arm: every rank but 0 leaves at once without work
    rc = bench.run_reference(A()) if rank != 0 else 0
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ws, r, local, t, rc))


def test_two_gloo_ranks_max_time_and_rank0_only_reference():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for rank, ws, r, local, t, rc in out:
        assert (ws, r, local) == (2, rank, rank)
        assert t == 2.5            # the slowest rank's time, on every rank
        assert rc == 0
