"""Multi-process coordination of bench.py's replicas (one process per GPU,
no data-path collective): barrier, max over ranks and the whole-job rate,
run as two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    import torch.distributed as dist
    ws, r, local = bench.dist_setup(2, backend="gloo")
    assert (ws, r, local) == (2, rank, rank)
    bench.barrier(ws)
    slowest = bench.max_over_ranks(ws, 10.0 + rank)  # rank 1 is slower
    rate = bench.aggregate_rate(ws, 1e9, 4, slowest)
    with open(os.path.join(out_dir, "r%d" % rank), "w") as f:
        f.write("%r %r" % (slowest, rate))
    dist.destroy_process_group()


def test_replicas_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        slowest, rate = open(tmp_path / ("r%d" % rank)).read().split()
        assert float(slowest) == 11.0
        # 2 ranks x 4 steps x 1 GB in 11 ms
        assert abs(float(rate) - 2 * 4 * 1e9 / 0.011 / 1e9) < 1e-6
