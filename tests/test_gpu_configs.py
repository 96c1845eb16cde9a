"""Parity at the benchmark sizes the small-case tests do not reach.

  * 128^3 k^-3 field, 100 isovalues, 256 bins, in full: every surface's
    counts, every distance field bit for bit, the FP64 ISM against the oracle
    over all 4950 pairs; brute force equals the LBVH on sampled surfaces.
  * 256^3 blobs + noise, 256 isovalues, 256 bins (the benchmark workload),
    on a stated sample: the whole pipeline runs, then 64 joint histograms
    spread over its segment-major chunks, 8 surfaces' vertex sets and 1 M
    sampled voxels of their distance fields are checked bit for bit.
  * 600 x 248 x 248 in the reference frame, where the reference's classify
    launch covers only part of the volume (MarchingCube.cpp:594-608).
  * A segment-major run with more pairs than one chunk holds.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-6
THREADS = 16


def engine_fields(ctx, rows, F):
    return np.stack([ctx.copy_field(int(r), np.zeros(F, np.float32)) for r in rows])


def oracle_map_f64(fields, bins, pairs):
    """FP64 NMI of the given (i, j) pairs over fields, in parallel."""
    iv = [oracle.field_interval(f) for f in fields]
    n = fields.shape[1]

    def one(p):
        i, j = p
        joint, _, _ = oracle.pair_histogram(fields[i], fields[j], bins, iv[i], iv[j])
        return oracle.mi_f64(joint, n)

    with ThreadPoolExecutor(THREADS) as ex:
        return np.array(list(ex.map(one, pairs)), np.float64)


def test_config2_full_size():
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config2()
    dims = (128, 128, 128)
    F = 128 ** 3
    with isosim.Context(0) as ctx:
        ism, ids, stats, _ = ctx.ism(vol.ravel(), dims, isos, df_method=isosim.DF_LBVH, bins=bins)
        fields = engine_fields(ctx, range(len(ids)), F)
        pts_all, _ = ctx.surface_points(vol.ravel(), dims, isos)
        # brute force on three surfaces: the same fields bit for bit
        for r in (0, len(ids) // 2, len(ids) - 1):
            pts = pts_all[ids[r]]
            bf = ctx.distance_field(oracle.normalize_points(pts, dims), dims, method=isosim.DF_BRUTE)
            assert np.array_equal(bf, fields[r]), r

    def surface(k):
        pts, active, total = oracle.marching_cubes(vol, dims, float(isos[k]), frame=0)
        assert stats[k].active_voxels == active and stats[k].total_verts == total and stats[k].points == len(pts)
        assert np.array_equal(pts_all[k], pts), k
        return oracle.distance_field_kd(oracle.normalize_points(pts, dims), dims) if len(pts) else None

    with ThreadPoolExecutor(THREADS) as ex:
        want = list(ex.map(surface, range(len(isos))))
    assert np.array_equal(ids, [k for k, f in enumerate(want) if f is not None])
    for r, k in enumerate(ids):
        assert np.array_equal(fields[r], want[k]), k
    m = len(ids)
    pairs = [(i, j) for i in range(m) for j in range(i + 1, m)]
    vals = oracle_map_f64(fields, bins, pairs)
    got = np.array([ism[i, j] for i, j in pairs], np.float64)
    assert np.abs(got - vals).max() < TOL
    assert np.array_equal(ism, ism.T)


def test_config3_sampled():
    """The 256^3 workload through the whole pipeline (REF32 mode keeps every
    pair's joint histogram on the device), checked on a sample."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config3()
    dims = (256, 256, 256)
    F = 256 ** 3
    rng = np.random.default_rng(3)
    with isosim.Context(0) as ctx:
        ism64, ids, stats, _ = ctx.ism(vol.ravel(), dims, isos, bins=bins)
        m = len(ids)
        assert m == 256
        ctx.set_mi_mode(isosim.MI_REF32)
        ism32, ids32, _, _ = ctx.ism(vol.ravel(), dims, isos, bins=bins)
        assert np.array_equal(ids, ids32)
        # 64 unordered pairs among 24 fields spread over the map, i.e. over
        # the segment-major chunks (4096 pairs each, 9 chunks)
        pool = np.sort(rng.choice(m, 24, replace=False))
        cand = [(int(pool[a]), int(pool[b])) for a in range(24) for b in range(a + 1, 24)]
        pairs = sorted(cand[q] for q in rng.choice(len(cand), 64, replace=False))
        rows = sorted({r for p in pairs for r in p})
        fields = dict(zip(rows, engine_fields(ctx, rows, F)))
        hists = {p: ctx.joint_histogram(p[0], p[1], bins) for p in pairs}
        hists_t = {p: ctx.joint_histogram(p[1], p[0], bins) for p in pairs[:8]}
        surf_k = [int(ids[r]) for r in rng.choice(m, 8, replace=False)]
        surf_fields = {k: ctx.copy_field(int(np.nonzero(ids == k)[0][0]), np.zeros(F, np.float32)) for k in surf_k}
        pts, _ = ctx.surface_points(vol.ravel(), dims, isos[surf_k])

    def pair(p):
        i, j = p
        joint, cs, rs = oracle.pair_histogram(fields[i], fields[j], bins)
        assert np.array_equal(hists[p], joint), p
        assert abs(ism64[i, j] - oracle.mi_f64(joint, F)) < TOL
        assert abs(ism32[i, j] - oracle.mi_f32(joint, cs, rs, F)) < 1e-5
        if p in hists_t:
            assert np.array_equal(hists_t[p], joint.T)
        return True

    with ThreadPoolExecutor(THREADS) as ex:
        assert all(ex.map(pair, pairs))

    sample = rng.choice(F, 1 << 20, replace=False)

    def surface(q):
        k = surf_k[q]
        want, _, _ = oracle.marching_cubes(vol, dims, float(isos[k]), frame=0)
        assert np.array_equal(pts[q], want), k
        df = oracle.distance_field_kd(oracle.normalize_points(want, dims), dims, idx=sample)
        assert np.array_equal(surf_fields[k][sample], df), k
        return True

    with ThreadPoolExecutor(8) as ex:
        assert all(ex.map(surface, range(8)))


def test_reference_frame_truncated_classify_grid():
    """600 x 248 x 248 = 36,902,400 voxels: the reference's classify launch
    covers 33,554,432 of them; vertex sets, active cells and triangle-vertex
    counts against the oracle's restatement of that launch."""
    import isosim
    import isosim.synth as synth
    dims = (600, 248, 248)
    vol = synth.gaussian_blobs(dims, 8, 5104, sigma=(4.0 * 248 / 64, 12.0 * 248 / 64))
    isos = synth.inside_isovalues(vol, 5)[1:4]
    with isosim.Context(0) as ctx:
        pts, stats = ctx.surface_points(vol.ravel(), dims, isos, frame=isosim.FRAME_REF)

    def one(q):
        want, active, total = oracle.marching_cubes(vol, dims, float(isos[q]), frame=0)
        assert stats[q].active_voxels == active and stats[q].total_verts == total, q
        assert np.array_equal(pts[q], want), q
        return len(want)

    with ThreadPoolExecutor(3) as ex:
        counts = list(ex.map(one, range(3)))
    assert min(counts) > 0


def test_segment_major_more_pairs_than_one_chunk():
    """91 fields (4186 unordered pairs) at 256 bins with 65,536-value
    segments: two chunks of per-pair histograms (4096 pairs fill 1 GB)."""
    import isosim
    rng = np.random.default_rng(91)
    n = 140001
    base = rng.uniform(0, 1, n)
    f = np.stack([np.abs(base * (1 + 0.02 * k) + 0.1 * rng.standard_normal(n)) for k in range(91)]).astype(np.float32)
    with isosim.Context(0) as ctx:
        ctx.set_hist_segment_values(65536)
        ism = ctx.similarity_map(f, 256)
        ctx.set_mi_mode(isosim.MI_REF32)
        ctx.similarity_map(f, 256)
        probe = [(0, 1), (3, 90), (44, 45), (80, 89), (89, 90), (17, 72)]
        hists = {p: ctx.joint_histogram(p[0], p[1], 256) for p in probe}
    for p, h in hists.items():
        want, _, _ = oracle.pair_histogram(f[p[0]], f[p[1]], 256)
        assert np.array_equal(h, want), p
    pairs = [(i, j) for i in range(91) for j in range(i + 1, 91)]
    vals = oracle_map_f64(f, 256, pairs)
    got = np.array([ism[i, j] for i, j in pairs], np.float64)
    assert np.abs(got - vals).max() < TOL
