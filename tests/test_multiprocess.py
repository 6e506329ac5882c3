"""The benchmark's multi-process path (replicas: one process per GPU, the
job's time the slowest rank's, the value all ranks' units over it) with two
gloo ranks on the CPU: rendezvous, max over ranks, barrier."""
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
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "CUDA_VISIBLE_DEVICES": ""})
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, dist = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank) and dist is not None
    assert dist.get_backend() == "gloo"
    # each rank's "time"; the job's time is the largest
    t = bench.max_over_ranks(dist, 1.0 + 2.5 * rank)
    bench.barrier(dist)
    units = 100.0 * w  # every replica did 100 units
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{t} {units / t}")
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    vals = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(2)]
    for t, v in vals:
        assert float(t) == 3.5  # max(1.0, 3.5) on every rank
        assert float(v) == pytest.approx(200.0 / 3.5)
    assert torch is not None
