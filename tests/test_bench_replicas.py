"""The replica path of bench.py on CPU: independent cubes per rank, the job's
time is the slowest rank's (max over ranks with gloo, world size 2), and the
value is the total particles over that time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [120.0, 95.5][rank]  # rank 1 is faster
        t = bench.max_over_ranks(local_ms, dist, device="cpu")
        out[rank] = (t, bench.replica_value(16_777_216, world, t * 1e-3))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_value_gloo():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 120.0  # both ranks see the slowest time
    assert res[0][1] == pytest.approx(2 * 16_777_216 / 0.120)


def test_single_rank_is_identity():
    assert bench.max_over_ranks(7.25) == 7.25
    assert bench.replica_value(1000, 1, 0.5) == 2000.0
