"""The multi-GPU form is replicas only: every rank evaluates its own box and the bench
reports the slowest rank's time.  This checks that host logic with two gloo ranks on the
CPU (no GPU, no data-path collective)."""
import os
import socket
import sys

import pytest

from conftest import REPO

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank, world, "cpu")
        torch.distributed.barrier()
        # the reference arm: rank 0 alone runs and prints, the other ranks do no work
        ref = bench.run_reference(None, rank, world) if rank != 0 else "rank0"
        out.put((rank, t, ref))
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_ranks_and_reference_arm_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == 2.5 and res[1][1] == 2.5
    assert res[1][2] is None
