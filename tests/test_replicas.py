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


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench as B
    t = B.reduce_over_ranks(1.5 + rank, "max")
    b = B.reduce_over_ranks(1000.0 * (rank + 1), "sum")
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{t} {b}")
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_times_and_bytes(tmp_path):
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)  # spawn, not fork
    for r in range(2):
        assert (tmp_path / f"rank{r}.txt").read_text() == "2.5 3000.0"


def test_single_process_is_the_identity():
    import bench as B
    assert B.reduce_over_ranks(3.25, "max") == 3.25
    assert B.reduce_over_ranks(7.0, "sum") == 7.0
