"""bench.py's multi-GPU path ("replicas only": every rank assembles its own
replica, the job's step time is the slowest rank's, the rate counts every
rank's entries), exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = [3.0, 5.5][rank]
        dist.barrier()
        slowest = bench.max_over_ranks(ms, device="cpu")
        out[rank] = (slowest, bench.job_rate(world, 297685449, slowest), bench.dist_env())
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 5.5
    # the job moves both replicas' entries per step of the slowest rank
    assert abs(res[0][1] - 2 * 297685449 / 5.5e-3 / 1e9) < 1e-9
    assert [res[r][2][:2] for r in (0, 1)] == [(0, 2), (1, 2)]


def test_single_process_is_its_own_maximum():
    import bench
    assert bench.max_over_ranks(4.25, device="cpu") == 4.25
    assert abs(bench.job_rate(1, 297685449, 3.2) - 93.0267) < 1e-3
