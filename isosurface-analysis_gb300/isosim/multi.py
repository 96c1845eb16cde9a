"""Multi-volume similarity batch across ranks (one process per GPU).

The reference splits this work across cluster jobs through files and merges
their JSON ledgers afterwards (runtime/src/Stitch.cpp:18-85).  Here the
volumes are sharded over ranks, each rank computes the ISMs and representative
distance fields of its own volumes, one all-gather gives every rank all
representative fields, each rank computes a contiguous share of the
cross-map blocks, and one gather brings the pair map to rank 0.  That
all-gather is the batch's only exchange.

The block list and the sharding are pure functions, so the same code runs on
GPUs (NCCL) and in CPU tests (gloo) with a CPU stand-in for the pair-map
kernel.
"""
import numpy as np


def cross_blocks(variables, timesteps):
    """Volume pairs of the reference's multi module (runtime/src/MultiVar.cpp:110-152):
    same variable across timesteps t1 < t2, and every variable pair at equal timestep.
    Volume id = var * timesteps + t."""
    blocks = []
    for v in range(variables):
        for t1 in range(timesteps):
            for t2 in range(t1 + 1, timesteps):
                blocks.append((v * timesteps + t1, v * timesteps + t2))
    for t in range(timesteps):
        for v1 in range(variables):
            for v2 in range(v1 + 1, variables):
                blocks.append((v1 * timesteps + t, v2 * timesteps + t))
    return blocks


def shard(count, rank, world):
    """Contiguous share [lo, hi) of `count` items for `rank`."""
    per = (count + world - 1) // world
    lo = min(rank * per, count)
    return lo, min(lo + per, count)


def block_pairs(blocks, reps):
    """Field pairs (rows of the representative matrix) of each volume block:
    block (a, b) gives (a*reps + i, b*reps + j) for i, j in [0, reps), i major."""
    if len(blocks) == 0:
        return np.empty((0, 2), dtype=np.int32)
    bl = np.asarray(blocks, dtype=np.int64).reshape(-1, 1, 1, 2)
    i = np.arange(reps).reshape(1, reps, 1)
    j = np.arange(reps).reshape(1, 1, reps)
    out = np.empty((len(blocks), reps, reps, 2), dtype=np.int32)
    out[..., 0] = bl[..., 0] * reps + i
    out[..., 1] = bl[..., 1] * reps + j
    return out.reshape(-1, 2)


def run_batch(dist, rank, world, variables, timesteps, reps, local_fields_fn, pair_map_fn):
    """Sharded batch over variables x timesteps volumes.

    Volume id = var * timesteps + t; rank r owns shard(volumes, r, world).
    local_fields_fn(vol_lo, vol_hi) -> tensor [(vol_hi-vol_lo)*reps, n] of this rank's
        representative fields (padded rows allowed: all ranks return the same width).
    pair_map_fn(fields [volumes*reps, n], pairs int32 [P, 2]) -> values float32 [P].
    Returns the full pair map [volumes*reps, volumes*reps] on rank 0 (None elsewhere)
    and the block list it covers."""
    import torch

    volumes = variables * timesteps
    lo, hi = shard(volumes, rank, world)
    mine = local_fields_fn(lo, hi)
    per = (volumes + world - 1) // world
    width = mine.shape[1]
    # equal-sized contributions: pad the last shard
    padded = torch.zeros((per * reps, width), dtype=mine.dtype, device=mine.device)
    padded[: mine.shape[0]] = mine
    gathered = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(gathered, padded)
    fields = torch.cat(gathered)[: volumes * reps]
    blocks = cross_blocks(variables, timesteps)
    blo, bhi = shard(len(blocks), rank, world)
    pairs = block_pairs(blocks[blo:bhi], reps)
    vals = pair_map_fn(fields, pairs)
    # gather every rank's values at rank 0 (padded to equal length)
    per_blocks = (len(blocks) + world - 1) // world
    buf = torch.zeros(per_blocks * reps * reps, dtype=torch.float32, device=mine.device)
    buf[: len(vals)] = torch.as_tensor(vals, dtype=torch.float32, device=mine.device)
    outs = [torch.empty_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, outs, dst=0)
    if rank != 0:
        return None, blocks
    R = volumes * reps
    full = np.zeros((R, R), dtype=np.float32)
    for r in range(world):
        b0, b1 = shard(len(blocks), r, world)
        p = block_pairs(blocks[b0:b1], reps)
        v = outs[r].cpu().numpy()[: len(p)]
        full[p[:, 0], p[:, 1]] = v
        full[p[:, 1], p[:, 0]] = v
    return full, blocks
