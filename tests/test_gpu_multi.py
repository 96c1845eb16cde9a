"""Batched cross maps over many volumes (one launch for every field pair of
every volume pair) and their block aggregation, against the oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_pair_map_and_blocks_match_oracle():
    import isosim
    import isosim.synth as synth
    dims = (20, 20, 20)
    k = 4
    vols = [synth.gaussian_blobs(dims, 4, 300 + v, sigma=(2.0, 5.0)) for v in range(3)]
    fields = []
    with isosim.Context(0) as ctx:
        F = dims[0] * dims[1] * dims[2]
        for vol in vols:
            isos = synth.inside_isovalues(vol, 12)
            ism, ids, _, _ = ctx.ism(vol.ravel(), dims, isos, bins=32)
            reps = isosim.select_representatives(ism, ids, isos, k)
            for r in sorted(x[3] for x in reps):
                fields.append(ctx.copy_field(r, np.zeros(F, np.float32)).copy())
        fields = np.stack(fields)
        R = fields.shape[0]
        blocks = [(0, 1), (0, 2), (1, 2), (1, 1)]
        pairs = [(a * k + i, b * k + j) for a, b in blocks for i in range(k) for j in range(k)]
        pmap = ctx.pair_map(fields, pairs, bins=32)
        agg = ctx.block_similarity(pmap, k, blocks)
    for a, b in pairs:
        joint, _, _ = oracle.pair_histogram(fields[a], fields[b], 32)
        want = oracle.mi_f64(joint, F)
        assert abs(pmap[a, b] - want) < 1e-6 and pmap[b, a] == pmap[a, b]
    for q, (a, b) in enumerate(blocks):
        blk = pmap[a * k:(a + 1) * k, b * k:(b + 1) * k].astype(np.float64)
        assert abs(agg[q, 0] - blk.mean()) < 1e-5
        best = 0.5 * (blk.max(axis=1).mean() + blk.max(axis=0).mean())
        assert abs(agg[q, 1] - best) < 1e-5


def test_cross_map_equals_pair_map_block():
    import isosim
    rng = np.random.default_rng(4)
    n = 30011
    a = np.abs(rng.standard_normal((3, n))).astype(np.float32)
    b = np.abs(rng.standard_normal((3, n)) * 2).astype(np.float32)
    with isosim.Context(0) as ctx:
        cm = ctx.cross_map(a, b, 64)
        allf = np.concatenate([a, b])
        pm = ctx.pair_map(allf, [(i, 3 + j) for i in range(3) for j in range(3)], bins=64)
    assert np.array_equal(cm, pm[:3, 3:])
