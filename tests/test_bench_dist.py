"""The bench's multi-rank host logic on CPU: two gloo ranks, max over ranks
of the step time, and the whole-job throughput of N replicas."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_info() == (ws, rank)
    ms = bench.max_over_ranks(100.0 * (rank + 1), dist)
    v = bench.job_throughput(ws, 1000, ms)
    with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
        f.write(f"{ms} {v}")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step(tmp_path):
    import torch.multiprocessing as mp
    ws = 2
    mp.spawn(_rank, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True)
    for r in range(ws):
        ms, v = map(float, open(tmp_path / f"r{r}").read().split())
        assert ms == 200.0                        # the slower rank's step
        assert v == pytest.approx(2 * 1000 / 0.2)  # labels of both replicas per second


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.job_throughput(1, 10, 1000.0) == 10.0
