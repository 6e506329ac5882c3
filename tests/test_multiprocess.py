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


# ---------------------------------------------------------------- sharding

def _sharding_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "CUDA_VISIBLE_DEVICES": ""})
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch.distributed as dist
    import oracle
    from opencal_gb300 import sharding as S
    from opencal_gb300 import workloads as W
    dist.init_process_group("gloo")
    res = {}
    # one grid by row slabs: Life (bytes, radius 1) and the neighbourhood
    # probe (FP64, Moore, radius 1), flat boundary, k steps between exchanges
    life0 = W.life_state(61, 45, p=0.35, seed=3)
    slabs = S.RowSlabs(61, world, k=3, radius=1)
    res["life"] = S.run_row_slabs(lambda a, n: oracle.life2d(a, n, toroidal=False), life0, 20, slabs, dist)
    v0 = W.random_field((50, 37), seed=5)
    slabs = S.RowSlabs(50, world, k=4, radius=1)
    res["probe"] = S.run_row_slabs(lambda a, n: oracle.nbprobe2d(a, n, nbhd=2, toroidal=False), v0, 13, slabs,
                                   dist)
    # instances: per-instance loss and central-difference gradient of
    # SCIDDICA-T by the oracle, for this rank's share only, then gathered
    dims = [(40, 36), (52, 30), (36, 44), (48, 48), (30, 40)]
    res["instances"] = S.sharded_map(lambda i: _instance_result(dims[i], i), [r * c for r, c in dims], dist)
    np.savez(os.path.join(out_dir, f"shard{rank}.npz"), **res)
    dist.destroy_process_group()


def _instance_result(dim, i):
    """Loss sum (h_T - h_target)^2 and its central differences in (p_r,
    p_eps) for instance i (the target from p_r = 0.42, p_eps = 0.0015)."""
    import numpy as np
    import oracle
    from opencal_gb300 import workloads as W
    z, h = W.sciddicaT_inputs(dim[0], dim[1], seed=700 + i, margin=8)
    tgt = oracle.sciddicaT(z, h, 25, p_r=0.42, p_eps=0.0015)[1]

    def loss(pr, pe):
        return float(np.sum((oracle.sciddicaT(z, h, 25, p_r=pr, p_eps=pe)[1] - tgt) ** 2))
    pr, pe, d = 0.5, 0.001, 1e-6
    return [loss(pr, pe), (loss(pr * (1 + d), pe) - loss(pr * (1 - d), pe)) / (2 * pr * d),
            (loss(pr, pe * (1 + d)) - loss(pr, pe * (1 - d))) / (2 * pe * d)]


@pytest.mark.parametrize("world", [2, 3])
def test_sharding_on_gloo_ranks(tmp_path, world, oracle_lib):
    """Row slabs with halo exchange give the whole grid's bits; instance
    sharding gathers every instance's loss and gradient in order, equal to
    the single-process result."""
    pytest.importorskip("torch")
    import numpy as np
    import torch.multiprocessing as mp
    from opencal_gb300 import workloads as W
    oracle = oracle_lib
    port = _free_port()
    mp.start_processes(_sharding_main, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    life_ref = oracle.life2d(W.life_state(61, 45, p=0.35, seed=3), 20, toroidal=False)
    probe_ref = oracle.nbprobe2d(W.random_field((50, 37), seed=5), 13, nbhd=2, toroidal=False)
    dims = [(40, 36), (52, 30), (36, 44), (48, 48), (30, 40)]
    inst_ref = np.array([_instance_result(d, i) for i, d in enumerate(dims)])
    for r in range(world):
        got = np.load(tmp_path / f"shard{r}.npz")
        assert got["life"].tobytes() == life_ref.tobytes()
        assert got["probe"].tobytes() == probe_ref.tobytes()
        assert got["instances"].tobytes() == inst_ref.tobytes()


def test_shard_instances_balances_cells():
    from opencal_gb300.sharding import RowSlabs, shard_instances
    assert shard_instances([10, 10, 10, 10], 2) == [(0, 2), (2, 4)]
    parts = shard_instances([100, 1, 1, 1, 100, 1], 3)
    assert parts[0][0] == 0 and parts[-1][1] == 6 and all(e > s for s, e in parts)
    assert shard_instances([5, 5], 3) == [(0, 1), (1, 2), (2, 2)]
    s = RowSlabs(20, 3, k=2, radius=2)
    assert s.owned == [(0, 6), (6, 13), (13, 20)]
    assert s.extended(0) == (0, 10) and s.extended(1) == (2, 17) and s.extended(2) == (9, 20)
    with pytest.raises(ValueError):
        RowSlabs(10, 4, k=3, radius=1)
