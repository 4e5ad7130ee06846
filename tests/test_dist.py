"""The multi-rank path of bench.py (one replica per GPU under torchrun) on CPU:
two gloo ranks, the barrier, the max over ranks and the whole-job rate."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WR_DIST_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    r, ws, local, tdist = bench._dist()
    assert (r, ws, local) == (rank, world, rank)
    bench._barrier(tdist)
    slowest = bench._max_over_ranks(tdist, 1.0 + rank)
    rate = bench.whole_job_rate(tdist, ws, 2, 1000, 2.0 + rank)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{slowest} {rate}\n")
    tdist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for rank in range(2):
        slowest, rate = map(float, (tmp_path / f"rank{rank}.txt").read_text().split())
        assert slowest == 2.0                       # max over ranks of 1.0, 2.0
        assert rate == 2 * 2 * 1000 / 3.0           # both ranks' cells over the slowest rank's time
