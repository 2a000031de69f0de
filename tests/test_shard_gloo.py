"""Multi-rank sharding of the pair output, on CPU with the gloo backend
(world_size 2).  Each rank computes its row range (here with the oracle, the
GPU path uses the same row-range arguments) and an all_gather reassembles the
matrix, which must equal the unsharded result exactly."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from cpptraj_gb300 import shard, synth


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, kind, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    X, m = synth.trajectory(17, 37, 40, 0.2, 1.5, np.float32, True)
    if kind == 0:
        ranges = shard.tri_row_ranges(X.shape[0], world)
        rb, re_ = ranges[rank]
        part = oracle.allpairs(X, tgt_mass=m, row_begin=rb, row_end=re_)
        total = oracle.n_out(X.shape[0], X.shape[0], 0)
    else:
        A, B = X[:15], X[15:]
        ranges = shard.full_row_ranges(B.shape[0], world)
        rb, re_ = ranges[rank]
        part = oracle.allpairs(A, B, tgt_mass=m, row_begin=rb, row_end=re_)
        total = oracle.n_out(A.shape[0], B.shape[0], 1)
    sizes = [None] * world
    dist.all_gather_object(sizes, int(part.size))
    buf = torch.zeros(max(sizes), dtype=torch.float32)
    buf[: part.size] = torch.from_numpy(part)
    gathered = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(gathered, buf)
    if rank == 0:
        full = np.concatenate([g[:s].numpy() for g, s in zip(gathered, sizes)])
        q.put((full.size == total, full))
    dist.destroy_process_group()


@pytest.mark.parametrize("kind", [0, 1])
def test_two_rank_shards_reassemble(kind):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, kind, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, full = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    X, m = synth.trajectory(17, 37, 40, 0.2, 1.5, np.float32, True)
    ref = oracle.allpairs(X, tgt_mass=m) if kind == 0 else oracle.allpairs(X[:15], X[15:], tgt_mass=m)
    assert ok
    assert np.array_equal(full, ref)


def test_tri_ranges_balanced():
    n = 1000
    rs = shard.tri_row_ranges(n, 4)
    assert rs[0][0] == 0 and rs[-1][1] == n
    counts = [shard.tri_elements_before(n, b) - shard.tri_elements_before(n, a) for a, b in rs]
    assert max(counts) - min(counts) <= n
    assert all(rs[k][1] == rs[k + 1][0] for k in range(3))
