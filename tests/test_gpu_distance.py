"""Distance fields on the GPU: brute force and LBVH are bit-identical to the
oracle's canonical FP32 field and within 4 float ulps (relative) of the exact
FP64 nearest distance."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def check(ctx, pts_norm, dims, ds=1):
    import isosim
    want = oracle.distance_field_f32(pts_norm, dims, ds)
    exact = oracle.distance_field_f64(pts_norm, dims, ds)
    for method in (isosim.DF_BRUTE, isosim.DF_LBVH):
        got = ctx.distance_field(pts_norm, dims, ds, method)
        assert np.array_equal(got, want), (method, np.abs(got - want).max())
    if len(pts_norm) > 1:
        err = np.abs(want.astype(np.float64) - exact)
        assert np.all(err <= 4 * np.spacing(np.maximum(exact, 1e-30).astype(np.float32)).astype(np.float64) + 1e-12)


@pytest.mark.parametrize("P", [2, 3, 17, 1000, 5000])
def test_random_points(ctx, P):
    rng = np.random.default_rng(P)
    check(ctx, rng.uniform(0, 1, (P, 3)).astype(np.float32), (20, 18, 16))


def test_single_point_stores_squared_distance(ctx):
    p = np.array([[0.3, 0.5, 0.7]], np.float32)
    check(ctx, p, (10, 10, 10))
    got = ctx.distance_field(p, (10, 10, 10))
    s = np.float32(np.float32(0) / np.float32(10))
    d0 = np.float32(s - p[0, 0]) ** 2
    assert got[0] == oracle.distance_field_f32(p, (10, 10, 10))[0]
    assert got[0] > 0.2  # squared, not sqrt (~0.91^2)


def test_duplicate_and_grid_points(ctx):
    """Integer cells (voxel approximation) normalised by the largest dimension:
    many equal Morton codes and many exact distance ties."""
    rng = np.random.default_rng(9)
    cells = rng.integers(0, 24, (3000, 3)).astype(np.float32)
    cells = np.concatenate([cells, cells[:500]])  # exact duplicates
    check(ctx, oracle.normalize_points(cells, (24, 24, 24)), (24, 24, 24))
    same = np.repeat(np.array([[0.5, 0.25, 0.125]], np.float32), 64, axis=0)
    check(ctx, same, (12, 12, 12))


@pytest.mark.parametrize("ds", [2, 3])
def test_downscale(ctx, ds):
    rng = np.random.default_rng(ds)
    check(ctx, rng.uniform(0, 1, (700, 3)).astype(np.float32), (24, 21, 18), ds)


def test_marching_cubes_points(ctx):
    import isosim.synth as synth
    dims = (28, 28, 28)
    vol = synth.gaussian_blobs(dims, 4, 8, sigma=(3.0, 6.0))
    iso = float(np.float32(vol.max() * 0.4))
    pts, _, _ = oracle.marching_cubes(vol, dims, iso, frame=0)
    check(ctx, oracle.normalize_points(pts, dims), dims)


def test_reference_named_entry():
    import isosim
    rng = np.random.default_rng(1)
    p = rng.uniform(0, 1, (900, 3)).astype(np.float32)
    assert np.array_equal(isosim.generate_hierarchy_h(p, (16, 16, 16)), oracle.distance_field_f32(p, (16, 16, 16)))


def test_lbvh_groups_beyond_256_surfaces(ctx):
    """More than 256 surfaces: the LBVH is built in groups of at most 256
    surfaces, whose sort keys carry 8 Morton bits per axis (the first group)
    and 9 (the rest); every field equals the brute-force field bit for bit."""
    import isosim
    import isosim.synth as synth
    dims = (24, 22, 20)
    vol = synth.gaussian_blobs(dims, 5, 3, sigma=(2.0, 5.0))
    lo, hi = float(vol.min()), float(vol.max())
    iso = np.linspace(lo, hi, 302)[1:-1].astype(np.float32)  # 300 isovalues strictly inside
    F = dims[0] * dims[1] * dims[2]
    got = {}
    for method in (isosim.DF_LBVH, isosim.DF_BRUTE):
        _, ids, _, _ = ctx.ism(vol.ravel(), dims, iso, df_method=method, bins=64)
        rows = np.zeros((len(ids), F), np.float32)
        for r in range(len(ids)):
            ctx.copy_field(r, rows[r])
        got[method] = (ids.copy(), rows)
    assert len(got[isosim.DF_LBVH][0]) > 256
    assert np.array_equal(got[isosim.DF_LBVH][0], got[isosim.DF_BRUTE][0])
    assert np.array_equal(got[isosim.DF_LBVH][1], got[isosim.DF_BRUTE][1])
