"""Tensor-core distance fields (ISO_DF_TC) against the exact methods.

The contraction only selects candidates; every field value is an exact FP32
distance, so the fields must equal the brute-force and LBVH fields bit for
bit, including the cases that stress the selection: near-ties (a sample at the
centre of a sphere of points), points a few ulps from samples, single-point
surfaces (squared distance), partial point blocks and bricks that overhang the
grid."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def fields_all_methods(ctx, pts_norm, dims, ds=1):
    import isosim
    return [ctx.distance_field(pts_norm, dims, downscale=ds, method=m)
            for m in (isosim.DF_TC, isosim.DF_BRUTE, isosim.DF_LBVH)]


@pytest.mark.parametrize("dims,ds", [((20, 18, 16), 1), ((24, 24, 24), 2), ((13, 31, 9), 1)])
def test_surfaces_bit_exact(ctx, dims, ds):
    import isosim.synth as synth
    vol = synth.gaussian_blobs(dims, 4, 91, sigma=(2.0, 5.0))
    for iso in synth.inside_isovalues(vol, 4):
        pts, _, _ = oracle.marching_cubes(vol, dims, float(iso), frame=0)
        if len(pts) == 0:
            continue
        pn = oracle.normalize_points(pts, dims)
        tc, bf, lb = fields_all_methods(ctx, pn, dims, ds)
        assert np.array_equal(tc, bf) and np.array_equal(tc, lb)
        assert np.array_equal(tc, oracle.distance_field_f32(pn, dims, ds))


@pytest.mark.parametrize("P", [1, 2, 255, 256, 257, 1000])
def test_point_counts(ctx, P):
    rng = np.random.default_rng(P)
    dims = (16, 16, 16)
    pts = rng.uniform(0, 1, (P, 3)).astype(np.float32)
    tc, bf, _ = fields_all_methods(ctx, pts, dims)
    assert np.array_equal(tc, bf)


def test_near_ties_on_a_sphere(ctx):
    """Points on a sphere around the centre sample: at that sample every point
    is a near-tie, and the minimum must still be the exact one."""
    rng = np.random.default_rng(5)
    dims = (16, 16, 16)
    v = rng.standard_normal((4000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    pts = (0.5 + 0.3 * v).astype(np.float32)
    tc, bf, lb = fields_all_methods(ctx, pts, dims)
    assert np.array_equal(tc, bf) and np.array_equal(tc, lb)


def test_points_next_to_samples(ctx):
    """Points a few ulps from sample positions and exactly on them: distances
    near and at zero."""
    dims = (16, 16, 16)
    g = (np.arange(16, dtype=np.float32) / np.float32(16))
    base = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)[::7]
    rng = np.random.default_rng(9)
    ulps = rng.integers(-3, 4, base.shape).astype(np.int32)
    near = (base.view(np.int32) + ulps).view(np.float32)
    pts = np.concatenate([near, base[::5]]).astype(np.float32)
    tc, bf, _ = fields_all_methods(ctx, pts, dims)
    assert np.array_equal(tc, bf)


def test_config1_pipeline(ctx):
    """The 64^3, 32-isovalue pipeline with tensor-core fields: same ISM and
    fields as the LBVH, bit for bit."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config1()
    a, ids, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, df_method=isosim.DF_TC, bins=bins)
    fa = [ctx.copy_field(r, np.zeros(64 ** 3, np.float32)) for r in range(len(ids))]
    b, ids2, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, df_method=isosim.DF_LBVH, bins=bins)
    fb = [ctx.copy_field(r, np.zeros(64 ** 3, np.float32)) for r in range(len(ids2))]
    assert np.array_equal(ids, ids2) and np.array_equal(a, b)
    for x, y in zip(fa, fb):
        assert np.array_equal(x, y)


def test_config2_sampled_surfaces(ctx):
    """Three surfaces of the 128^3 k^-3 field (tens of thousands of points)."""
    import isosim
    import isosim.synth as synth
    vol, isos, _ = synth.config2()
    dims = (128, 128, 128)
    pts, _ = ctx.surface_points(vol.ravel(), dims, isos[[10, 50, 90]])
    for p in pts:
        pn = oracle.normalize_points(p, dims)
        tc = ctx.distance_field(pn, dims, method=isosim.DF_TC)
        lb = ctx.distance_field(pn, dims, method=isosim.DF_LBVH)
        assert np.array_equal(tc, lb)
