"""CPU: the multi-process replica path of bench.py (one process per GPU, replicas only) on
world_size 2 with the gloo backend: rendezvous on 127.0.0.1, barrier, max-over-ranks timing."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    bench.barrier(w)
    # each replica times its own full workload; the job's time is the slowest rank's
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, w)
    out.put((rank, ms))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the CPU path is tested where no GPU is present")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 15.0), (1, 15.0)]
