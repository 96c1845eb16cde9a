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
(FRAME_REF).
"""
import numpy as np
import pytest

import oracle
import refgpu

pytestmark = pytest.mark.gpu

# generateTriangles' grid is halved in x while above 65535 blocks of 32
# (MarchingCube.cpp:674-678); with an odd block count the halving drops the
# last blocks, so surfaces above this many active voxels may lose vertices in
# the reference.  The workloads here stay below it (asserted).
HALVING_FREE = 65535 * refgpu.MC_NTHREADS


@pytest.fixture(scope="module", autouse=True)
def need_cubin():
    if not refgpu.mc_available():
        pytest.skip("reference cubin (oracle/_ref/ref_mc.cubin) not built")


def check_surfaces(vol, dims, isos):
    import isosim
    with isosim.Context(0) as ctx:
        pts, stats = ctx.surface_points(vol.ravel(), dims, isos, frame=isosim.FRAME_REF)
    nonempty = 0
    for q, iso in enumerate(isos):
        ref, active, total = refgpu.marching_cubes(vol.ravel(), dims, float(iso))
        assert active < HALVING_FREE, (q, active)
        want, o_active, o_total = oracle.marching_cubes(vol, dims, float(iso), frame=0)
        assert (o_active, o_total) == (active, total), q
        assert np.array_equal(want, ref), q
        assert stats[q].active_voxels == active and stats[q].total_verts == total, q
        assert np.array_equal(pts[q], ref), q
        nonempty += len(ref) > 0
    return nonempty


def test_blobs_64():
    """64^3 Gaussian blobs, all 32 isovalues of the workload."""
    import isosim.synth as synth
    vol, isos, _ = synth.config1()
    assert check_surfaces(vol, (64, 64, 64), isos) == len(isos)


def test_power_law_128():
    """128^3 k^-3 field, every fifth of its 100 isovalues."""
    import isosim.synth as synth
    vol, isos, _ = synth.config2()
    assert check_surfaces(vol, (128, 128, 128), isos[::5]) > 0


def test_blobs_256():
    """256^3 blobs + noise (the benchmark volume): the classify grid is
    reshaped to 32768 x 4 blocks; eight isovalues across its range."""
    import isosim.synth as synth
    vol, isos, _ = synth.config3()
    assert check_surfaces(vol, (256, 256, 256), isos[::32]) == 8


def test_truncated_classify_grid():
    """600 x 248 x 248: the reference's classify launch covers 33,554,432 of
    the 36,902,400 voxels; the rest stay unclassified in all three."""
    import isosim.synth as synth
    dims = (600, 248, 248)
    vol = synth.gaussian_blobs(dims, 8, 5104, sigma=(4.0 * 248 / 64, 12.0 * 248 / 64))
    isos = synth.inside_isovalues(vol, 5)[1:4]
    assert check_surfaces(vol, dims, isos) == 3


def test_ragged_volume():
    """A volume whose voxel count is not a multiple of the 128-thread block
    (61 x 37 x 29): the last V mod 128 voxels are not classified."""
    rng = np.random.default_rng(29)
    dims = (61, 37, 29)
    vol = rng.standard_normal(dims[::-1]).astype(np.float32)
    assert (dims[0] * dims[1] * dims[2]) % 128 != 0
    assert check_surfaces(vol, dims, np.array([-0.5, 0.0, 0.7], np.float32)) == 3
