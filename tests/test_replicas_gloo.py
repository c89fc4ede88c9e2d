"""Multi-process path of bench.py on CPU: the benchmark runs independent
replicas (the path does not shard across GPUs here), one per rank; the timed
region is the max over ranks and the value is the whole-job rate. Checked with
two gloo ranks on 127.0.0.1."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [120.0, 150.0][rank]
    m = bench.reduce_max_ms(ms, world, "cpu")
    out.put((rank, m, bench.replica_value(6, world, m)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_max_time_and_job_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]
    assert all(abs(r[2] - 12 / 0.150) < 1e-9 for r in res)


def test_single_process_is_identity():
    import bench
    assert bench.reduce_max_ms(42.0, 1) == 42.0
    assert bench.replica_value(3, 1, 1000.0) == 3.0
