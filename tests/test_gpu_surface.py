"""Surface extraction on the GPU against the oracle: marching-cubes vertex sets
bit-exact (reference and canonical frames), active-cell and triangle-vertex
counts exact; voxel approximation cells exact and in the reference's order."""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def blobs(dims, seed):
    import isosim.synth as synth
    return synth.gaussian_blobs(dims, 5, seed, sigma=(2.0, 5.0))


def check_mc(ctx, vol, dims, isos, frame):
    pts, stats = ctx.surface_points(vol.ravel(), dims, isos, surface=0, frame=frame)
    for k, iso in enumerate(isos):
        want, active, total = oracle.marching_cubes(vol, dims, float(iso), frame=frame)
        assert np.array_equal(pts[k], want), (k, iso, len(pts[k]), len(want))
        assert stats[k].active_voxels == active and stats[k].total_verts == total


@pytest.mark.parametrize("frame", [0, 1])
def test_mc_blobs(ctx, frame):
    dims = (24, 24, 24)
    vol = blobs(dims, 1)
    isos = np.linspace(vol.min(), vol.max(), 9)[1:-1].astype(np.float32)
    check_mc(ctx, vol, dims, isos, frame)


@pytest.mark.parametrize("frame", [0, 1])
def test_mc_many_clustered_isovalues(ctx, frame):
    """80 isovalues in no order, with ten equal ones and forty within 1e-4 of
    the range (many in one bucket of the searches' index), and the extremes
    of the range: vertex sets and counts exact."""
    dims = (20, 18, 16)
    vol = blobs(dims, 7)
    lo, hi = float(vol.min()), float(vol.max())
    rng = np.random.default_rng(11)
    c = lo + 0.3 * (hi - lo)
    isos = np.concatenate([rng.uniform(lo, hi, 28), [lo, hi], c + rng.uniform(0, 1e-4 * (hi - lo), 40),
                           np.full(10, c)]).astype(np.float32)
    rng.shuffle(isos)
    check_mc(ctx, vol, dims, isos, frame)


@pytest.mark.parametrize("frame", [0, 1])
def test_mc_noncubic_noise(ctx, frame):
    dims = (17, 13, 9)
    vol = np.random.default_rng(4).standard_normal(dims).astype(np.float32)
    check_mc(ctx, vol, dims, np.array([-0.7, 0.0, 0.2, 1.1], np.float32), frame)


@pytest.mark.parametrize("frame", [0, 1])
def test_mc_write_pass_counts_again(ctx, frame):
    """With no room for the per-block count table the write pass counts the
    vertex versions again: the same exact vertex sets and statistics."""
    import isosim
    dims = (40, 33, 29)
    vol = blobs(dims, 7) + 0.05 * np.random.default_rng(8).standard_normal(dims).astype(np.float32)
    isos = np.linspace(vol.min(), vol.max(), 12)[1:-1].astype(np.float32)
    c2 = isosim.Context(0)
    try:
        c2.set_surf_block_count_bytes(0)
        check_mc(c2, vol, dims, isos, frame)
    finally:
        c2.close()


def test_mc_integer_data_corner_vertices(ctx):
    """Isovalues equal to data values put vertices exactly on grid points that
    several edges share: the de-duplication must merge them."""
    dims = (12, 10, 11)
    vol = np.random.default_rng(5).integers(0, 5, dims).astype(np.float32)
    check_mc(ctx, vol, dims, np.array([1.0, 2.0, 2.5, 4.0], np.float32), 0)
    check_mc(ctx, vol, dims, np.array([1.0, 3.0], np.float32), 1)


def test_mc_reference_classification_limit(ctx):
    """V not a multiple of 128: the reference classifies only the first
    128*floor(V/128) voxels; the tail cells contribute nothing."""
    dims = (9, 7, 5)  # 315 voxels -> 256 classified
    assert oracle.orc.orc_mc_classified_voxels(315) == 256
    vol = np.random.default_rng(6).standard_normal(dims).astype(np.float32)
    check_mc(ctx, vol, dims, np.array([0.0, 0.5], np.float32), 0)


def test_mc_all_case_codes(ctx):
    counts = oracle.mc_vertex_counts()
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for case in range(256):
        vol = np.zeros((3, 3, 3), np.float32) + 2.0
        for k, (a, b, c) in enumerate(corner):
            vol[a, b, c] = 0.0 if (case >> k) & 1 else 1.0
        check_mc(ctx, vol, (3, 3, 3), np.array([0.5], np.float32), 1)


def test_approximation_golden_and_random(ctx):
    g = np.load(os.path.join(GOLDEN, "approx_small.npz"))
    dims = tuple(int(d) for d in g["dims"])
    pts, _ = ctx.surface_points(g["vol"].ravel(), dims, g["isos"], surface=1)
    off = 0
    for k, cnt in enumerate(g["counts"]):
        assert np.array_equal(pts[k].astype(np.int32), g["cells"][off:off + cnt])
        off += cnt
    dims = (30, 20, 25)
    vol = blobs(dims, 2)
    isos = np.linspace(vol.min(), vol.max(), 6)[1:-1].astype(np.float32)
    pts, _ = ctx.surface_points(vol.ravel(), dims, isos, surface=1)
    for k, iso in enumerate(isos):
        assert np.array_equal(pts[k].astype(np.int32), oracle.approximation(vol, dims, float(iso)))


def test_reference_named_surface_entries():
    import isosim
    dims = (32, 30, 28)
    vol = blobs(dims, 3)
    iso = float(np.float32((vol.min() + vol.max()) / 2))
    cells = isosim.approximate_isosurfaces_h(vol.ravel(), dims, iso)
    assert np.array_equal(cells, oracle.approximation(vol, dims, iso))
    v4 = isosim.marching_cube_h(vol.ravel(), dims, iso)
    want, _, total = oracle.marching_cubes(vol, dims, iso, frame=0)
    assert total <= dims[0] * dims[1] * dims[2] - 3
    assert np.array_equal(v4[:, :3], want) and np.all(v4[:, 3] == 1.0)


def test_marching_cube_entry_reports_reference_truncation():
    """Beyond maxVerts-3 triangle vertices the reference drops triangles and
    lets unwritten slots into its vertex set; the C entry refuses instead."""
    import isosim
    dims = (10, 10, 10)
    vol = np.random.default_rng(8).standard_normal(dims).astype(np.float32)
    _, _, total = oracle.marching_cubes(vol, dims, 0.0, frame=0)
    assert total > 1000 - 3
    with pytest.raises(isosim.IsoError) as e:
        isosim.marching_cube_h(vol.ravel(), dims, 0.0)
    assert e.value.code == isosim.ISO_ERR_CAPACITY
    pts, stats = isosim.Context(0).surface_points(vol.ravel(), dims, [0.0])
    assert stats[0].flags & isosim.MC_REF_DROPPED


def test_empty_and_out_of_range(ctx):
    dims = (8, 8, 8)
    vol = blobs(dims, 4)
    pts, stats = ctx.surface_points(vol.ravel(), dims, np.array([vol.max() + 1, vol.min() - 1], np.float32))
    assert all(len(p) == 0 for p in pts) and all(s.points == 0 for s in stats)
