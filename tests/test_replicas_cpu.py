"""The multi-GPU path of the benchmark: the reference has no domain
decomposition, so N GPUs run N independent replicas and the only collective
is the timing reduction.  Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    units = 1000 * (rank + 1)          # each replica's particle-pushes
    ms = 10.0 + 5.0 * rank             # each replica's time
    value, tmax = bench.replica_throughput(units, ms, ws, device="cpu")
    out[rank] = (value, tmax)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_aggregate_with_gloo():
    ws = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(ws, port, out), nprocs=ws, join=True, start_method="spawn")
        res = dict(out)
    # total units 3000 over the slowest rank's 15 ms
    for rank in range(ws):
        value, tmax = res[rank]
        assert tmax == 15.0
        assert abs(value - 3000 / 0.015) < 1e-6


def test_single_replica_is_plain_throughput():
    import bench
    value, ms = bench.replica_throughput(500, 20.0, 1)
    assert ms == 20.0 and abs(value - 25000.0) < 1e-9
