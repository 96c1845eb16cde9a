"""The engine's and the oracle's marching cubes against the reference's own
marching-cubes kernels.

oracle/build_ref.sh compiles the reference's MarchingCube.cu (device code,
nvcc default flags) into oracle/_ref/ref_mc.cubin; oracle/refgpu.py runs its
classifyVoxel, compactVoxels and generateTriangles on this GPU with the host
steps of cudaMarchingCube (MarchingCube.cpp:588-710): the truncated classify
grid, the vertex and occupancy scans, the grid halving of the triangle
launch, and the sort + unique of the emitted vertices.

Bar: the sorted, unique vertex set, the active-voxel count and the
triangle-vertex count of each surface are equal, bit for bit, between the
reference's kernels, the oracle (frame 0, the reference frame) and the engine
(FRAME_REF).  Two reference behaviours are documented exceptions, where the
reference leaves entries of its vertex buffer unwritten and sorts their zeros
into its vertex set:
  * more than maxVerts - 3 triangle vertices (maxVerts = the voxel count,
    Isosurface.cpp:263): only the triangles below that index are written
    (MarchingCube.cu:319); the engine flags the surface ISO_MC_REF_DROPPED;
  * more than 2,097,120 active voxels: the triangle launch's grid halving
    (MarchingCube.cpp:674-678) can drop the last blocks of 32 voxels; the
    engine emits every active voxel.
There the counts must still agree, every position the reference did write
must be a vertex of the engine's set, and (for the halving) the engine's set
may exceed it by at most the 12 edge vertices of each dropped voxel.
"""
import numpy as np
import pytest

import oracle
import refgpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_cubin():
    if not refgpu.mc_available():
        pytest.skip("reference cubin (oracle/_ref/ref_mc.cubin) not built")


def check_surfaces(vol, dims, isos):
    import isosim
    with isosim.Context(0) as ctx:
        pts, stats = ctx.surface_points(vol.ravel(), dims, isos, frame=isosim.FRAME_REF)
    V = dims[0] * dims[1] * dims[2]
    nonempty = dropped = 0
    for q, iso in enumerate(isos):
        ref4, active, total = refgpu.marching_cubes(vol.ravel(), dims, float(iso), with_w=True)
        want, o_active, o_total = oracle.marching_cubes(vol, dims, float(iso), frame=0)
        assert (o_active, o_total) == (active, total), q
        assert stats[q].active_voxels == active and stats[q].total_verts == total, q
        assert np.array_equal(pts[q], want), q
        overflow = total > V - 3
        assert bool(stats[q].flags & isosim.MC_REF_DROPPED) == overflow, q
        missed = active - refgpu.mc_generated_voxels(active)
        if overflow or missed:
            written = ref4[ref4[:, 3] == 1.0, :3]
            assert len(written) > 0 and len(written) <= len(want), q
            rows = want.view(np.dtype((np.void, 12))).ravel()
            assert np.isin(np.ascontiguousarray(written).view(np.dtype((np.void, 12))).ravel(), rows).all(), q
            if not overflow:
                assert len(want) - len(written) <= 12 * missed, q
            dropped += 1
        else:
            assert np.all(ref4[:, 3] == 1.0), q
            assert np.array_equal(want, ref4[:, :3]), q
        nonempty += len(want) > 0
    return nonempty, dropped


def test_blobs_64():
    """64^3 Gaussian blobs, all 32 isovalues of the workload."""
    import isosim.synth as synth
    vol, isos, _ = synth.config1()
    assert check_surfaces(vol, (64, 64, 64), isos) == (len(isos), 0)


def test_power_law_128():
    """128^3 k^-3 field, every fifth of its 100 isovalues; the ones near 0
    have more triangle vertices than voxels (the reference's overflow)."""
    import isosim.synth as synth
    vol, isos, _ = synth.config2()
    nonempty, dropped = check_surfaces(vol, (128, 128, 128), isos[::5])
    assert nonempty == 20 and dropped > 0


def test_blobs_256():
    """256^3 blobs + noise (the benchmark volume): the classify grid is
    reshaped to 32768 x 4 blocks; eight isovalues across its range, the
    second with 3.6 M active voxels (the triangle launch's halving)."""
    import isosim.synth as synth
    vol, isos, _ = synth.config3()
    nonempty, dropped = check_surfaces(vol, (256, 256, 256), isos[::32])
    assert nonempty == 8 and dropped >= 1


def test_truncated_classify_grid():
    """600 x 248 x 248: the reference's classify launch covers 33,554,432 of
    the 36,902,400 voxels; the rest stay unclassified in all three."""
    import isosim.synth as synth
    dims = (600, 248, 248)
    vol = synth.gaussian_blobs(dims, 8, 5104, sigma=(4.0 * 248 / 64, 12.0 * 248 / 64))
    isos = synth.inside_isovalues(vol, 5)[1:4]
    assert check_surfaces(vol, dims, isos)[0] == 3


def test_ragged_volume():
    """A volume whose voxel count is not a multiple of the 128-thread block
    (61 x 37 x 29): the last V mod 128 voxels are not classified."""
    import isosim.synth as synth
    dims = (61, 37, 29)
    assert (dims[0] * dims[1] * dims[2]) % 128 != 0
    vol = synth.gaussian_blobs(dims, 4, 29, sigma=(3.0, 6.0))
    assert check_surfaces(vol, dims, synth.inside_isovalues(vol, 5)[1:4]) == (3, 0)


def test_white_noise_overflow():
    """White noise on the same ragged grid: every surface has more triangle
    vertices than voxels, the reference's overflow in each."""
    rng = np.random.default_rng(29)
    dims = (61, 37, 29)
    vol = rng.standard_normal(dims[::-1]).astype(np.float32)
    assert check_surfaces(vol, dims, np.array([-0.5, 0.0, 0.7], np.float32)) == (3, 3)
