"""
Multi-process path on CPU (gloo, world size 2): instances shard across
ranks with no collective on the data path, and gathering the ranks' results
reproduces a single-process run.  The per-instance work here is the CPU
oracle (the GPU kernel's shard is the same index range).
"""

import os

import numpy as np
import pytest

from tvb_hpc import engine


def test_shard_partitions():
    for n in (0, 1, 7, 32, 4096, 4097):
        for world in (1, 2, 3, 8):
            got = [engine.shard(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [hi - lo for lo, hi in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        engine.shard(4, 2, 2)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import pyoracle as orc
    from tvb_hpc import network
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    w, ln = network.synthetic_connectome(20, 0.3, seed=0)
    c = network.Connectivity.from_dense(w, ln)
    I = 5
    rng = np.random.default_rng(0)
    x0 = rng.uniform(0, 6, (I, 20, 1)).astype(np.float32)
    G = np.linspace(0.1, 2, I).astype(np.float32)
    d = c.delays(4.0, 0.1, 'ceil')
    lo, hi = engine.shard(I, rank, world)
    res = orc.run(0, 2, c.row, c.col, c.wnz, 512, 200, 0.1, np.broadcast_to(d, (hi - lo, d.size)),
                  G[lo:hi], np.full((hi - lo, 20), 0.06, np.float32), x0[lo:hi],
                  inst_ids=np.arange(lo, hi))['state'] if hi > lo else np.zeros((0, 20, 1))
    parts = [None] * world
    dist.all_gather_object(parts, (lo, res))
    if rank == 0:
        full = np.concatenate([p[1] for p in sorted(parts, key=lambda p: p[0])])
        ref = orc.run(0, 2, c.row, c.col, c.wnz, 512, 200, 0.1, np.broadcast_to(d, (I, d.size)), G,
                      np.full((I, 20), 0.06, np.float32), x0)['state']
        np.save(out, np.abs(full - ref).max())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_replicas(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / 'err.npy')
    port = 29500 + (os.getpid() % 1000)
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert float(np.load(out)) == 0.0
