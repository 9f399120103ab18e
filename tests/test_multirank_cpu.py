"""Multi-rank path of bench.py on CPU: two gloo ranks, each with its own shard
of tissues, combined by the same reduction the GPU run uses (the slowest
rank's time, the sum of all ranks' vertex-steps).  Tissues are independent,
so the shards exchange nothing while stepping; only this reduction crosses
ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        # each rank's shard is seeded by its rank, as in bench.run_ours
        shard = bench.workload_batched(bench.OracleGeometry(), seed=1000 + rank, ntissues=3)
        verts = sum(int(t["nv"].sum()) for t in shard)
        secs, units = bench.reduce_over_ranks(1.0 + rank, float(verts), world, "cpu")
        out[rank] = (secs, units, verts, float(shard[0]["xy"][0, 0]))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_gloo_ranks():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    verts = [res[r][2] for r in range(world)]
    for r in range(world):
        secs, units, _, _ = res[r]
        assert secs == 2.0                      # slowest rank
        assert units == float(sum(verts))       # every shard counted once
    # the shards differ (independent tissues per rank)
    assert res[0][3] != res[1][3]
