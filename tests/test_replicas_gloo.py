"""Multi-GPU runs are replicas (independent instance shards, no data-path
collective): the host logic of bench.py under torch.distributed with the gloo
backend, world_size 2, on the CPU -- shard selection, barrier, max / sum."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    r, w, d = bench.dist_init(ws)
    insts = bench.workload("sweep", 0, r)
    key = [(round(i["a_over_R"], 12), round(i["beta"], 12)) for i in insts]
    allkeys = [None] * w
    d.all_gather_object(allkeys, key)
    bench.barrier(d)
    mx = bench.allmax(d, float(r + 1))
    sm = bench.allsum(d, float(len(insts)))
    q.put((r, w, len(insts), allkeys, mx, sm))
    dist.destroy_process_group()


def test_two_replicas_take_disjoint_shards():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    out.sort()
    for r, w, n, allkeys, mx, sm in out:
        assert w == 2 and n == 128
        assert mx == 2.0 and sm == 256.0
        assert not set(allkeys[0]) & set(allkeys[1])  # independent shards
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from sqbem import workloads
    assert bench.workload("sweep", 0, 0) == workloads.sweep()  # rank 0 = the single-GPU set
