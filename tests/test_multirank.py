"""The multi-rank host logic of bench.py on CPU (gloo, world size 2): each
rank solves its own batch (distinct problem seeds, weak scaling), the timing
is the maximum over ranks and the reported value aggregates all ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, dist = bench.dist_init()
    specs = bench._rank_specs(3, r)
    key = [round(float(sp.bl.x.sum()), 12) + sp.nx for sp in specs]
    keys = [None] * w
    dist.all_gather_object(keys, key)
    t = bench.max_over_ranks(dist, 10.0 + 5.0 * r, device="cpu")
    q.put((r, w, keys, t, bench.aggregate_value(w, 3, 2, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, keys0, t0, v0), (r1, w1, keys1, t1, v1) = out
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert keys0 == keys1 and set(keys0[0]).isdisjoint(keys0[1])   # distinct batches per rank
    assert t0 == t1 == 15.0                                          # max over ranks
    assert v0 == v1 == pytest.approx(2 * 3 * 2 / 0.015)             # all ranks' solves over that time


def test_rank0_batch_is_the_benchmark_batch():
    sys.path.insert(0, ROOT)
    import bench
    from immersedlayers import workloads as W
    a = bench._rank_specs(4, 0)
    b = W.batch_specs(4)
    assert [s.nx for s in a] == [s.nx for s in b]
    assert all((x.bl.x == y.bl.x).all() for x, y in zip(a, b))
