"""The sharded multi-volume batch on two CPU ranks (gloo): the all-gather of
representative fields plus per-rank block shares must give the same pair map
as one rank computing everything.  The pair-map kernel is stood in for by the
oracle's FP64 NMI (this test runs without a GPU)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

V, T, REPS, N, BINS = 2, 3, 3, 4000, 16


def local_fields(lo, hi):
    import torch
    rows = []
    for vol in range(lo, hi):
        rng = np.random.default_rng(100 + vol)
        base = rng.uniform(0, 1, N)
        for r in range(REPS):
            rows.append(np.abs(base * (1 + 0.2 * r) + 0.1 * rng.standard_normal(N)))
    return torch.tensor(np.array(rows), dtype=torch.float32)


def pair_values(fields, pairs):
    import oracle
    f = fields.numpy()
    out = []
    for a, b in pairs:
        joint, _, _ = oracle.pair_histogram(f[a], f[b], BINS)
        out.append(oracle.mi_f64(joint, f.shape[1]))
    return np.array(out, np.float32)


def worker(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    sys.path[:0] = [os.path.join(root, "isosurface-analysis_gb300"), os.path.join(root, "oracle")]
    import torch.distributed as dist
    from isosim import multi
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    full, blocks = multi.run_batch(dist, rank, world, V, T, REPS, local_fields, pair_values)
    if rank == 0:
        q.put((full, blocks))
    dist.barrier()
    dist.destroy_process_group()


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_batch_matches_single_rank():
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "isosurface-analysis_gb300"))
    from isosim import multi
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full, blocks = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert blocks == multi.cross_blocks(V, T)
    fields = local_fields(0, V * T)
    pairs = multi.block_pairs(blocks, REPS)
    want = pair_values(fields, pairs)
    assert np.array_equal(full[pairs[:, 0], pairs[:, 1]], want)
    assert np.array_equal(full[pairs[:, 1], pairs[:, 0]], want)


def test_cross_blocks_match_reference_loops():
    from isosim import multi
    blocks = multi.cross_blocks(4, 50)
    assert len(blocks) == 4 * 50 * 49 // 2 + 50 * 6  # 4900 same-variable + 300 cross-variable maps
    assert len(set(blocks)) == len(blocks)
    for r in range(3):
        lo, hi = multi.shard(10, r, 3)
        assert 0 <= lo <= hi <= 10
    assert sum(multi.shard(10, r, 3)[1] - multi.shard(10, r, 3)[0] for r in range(3)) == 10


def test_block_pairs_layout():
    """Field pairs of each volume block, i major: block (a, b) gives rows
    (a*reps + i, b*reps + j) in the order of two nested loops over i, j."""
    from isosim import multi
    blocks = multi.cross_blocks(3, 4)
    reps = 5
    want = [(a * reps + i, b * reps + j) for a, b in blocks for i in range(reps) for j in range(reps)]
    got = multi.block_pairs(blocks, reps)
    assert got.dtype == np.int32 and got.shape == (len(want), 2)
    assert [tuple(p) for p in got.tolist()] == want
    assert multi.block_pairs([], reps).shape == (0, 2)
