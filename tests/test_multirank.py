"""The N > 1 path of bench.py on CPU: two gloo ranks, as torchrun would start them. Every rank
solves its own replica (the path has no exchange step on one GPU), so the only collective is
the replica aggregation: the slowest rank's time and the ranks' total work."""

import multiprocessing as mp
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms, work = bench.reduce_over_ranks(dist, [2.5, 4.0][rank], [100, 140][rank], "cpu")
        q.put((rank, ms, work))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_over_two_gloo_ranks():
    """Both ranks see max(time) and sum(work): value = total work / slowest time."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 4.0, 240.0), (1, 4.0, 240.0)]


def test_single_rank_aggregation_is_the_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_over_ranks(None, 3.0, 5) == (3.0, 5.0)


def test_reference_arm_other_ranks_exit_without_work(capsys):
    """Under torchrun only rank 0 runs the reference arm; the others print nothing."""
    sys.path.insert(0, str(ROOT))
    import bench

    bench.run_reference(None, 1, 2)
    assert capsys.readouterr().out == ""
