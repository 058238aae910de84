"""The multi-GPU form is replicas only: every rank splits its own inputs, no collective touches the
data path, and bench.py combines the ranks' figures (max of times, sum of bytes).  That combination
runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench as B
    t = B.reduce_over_ranks(1.5 + rank, "max")
    b = B.reduce_over_ranks(1000.0 * (rank + 1), "sum")
    out[rank] = (t, b)
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_times_and_bytes():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: (2.5, 3000.0), 1: (2.5, 3000.0)}


def test_single_process_is_the_identity():
    import bench as B
    assert B.reduce_over_ranks(3.25, "max") == 3.25
    assert B.reduce_over_ranks(7.0, "sum") == 7.0
