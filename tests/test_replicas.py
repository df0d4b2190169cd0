"""Replica logic for N > 1 on CPU: world_size 2 over gloo (127.0.0.1), no GPU needed."""
import os
import socket

import pytest

from conftest import import_gdt


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rep = import_gdt().replicas
    weights = [(n + 1) ** 2 for n in (64, 512, 128, 256, 512, 64, 256, 128)]
    parts = rep.partition_by_weight(weights, world)
    mine = parts[rank]
    units = sum(weights[i] for i in mine)
    local_ms = 10.0 + rank  # rank 1 is the slow one
    value, ms = rep.whole_job_throughput(units, local_ms)
    dist.barrier()
    q.put((rank, parts, units, value, ms))
    dist.destroy_process_group()


def test_two_rank_partition_and_throughput():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res.sort()
    parts0, parts1 = res[0][1], res[1][1]
    assert parts0 == parts1  # every rank computes the same split
    total = sum((n + 1) ** 2 for n in (64, 512, 128, 256, 512, 64, 256, 128))
    assert res[0][2] + res[1][2] == total
    assert sorted(parts0[0] + parts0[1]) == list(range(8))
    for r in res:
        assert r[4] == pytest.approx(11.0)  # max over ranks
        assert r[3] == pytest.approx(total / 0.011)
    # the split is balanced to within one heavy item
    assert abs(res[0][2] - res[1][2]) <= 513 ** 2


def test_partition_single_rank_keeps_everything():
    rep = import_gdt().replicas
    assert rep.partition_by_weight([3, 1, 2], 1) == [[0, 2, 1]]
