"""The engine's voxel approximation against the reference's own kernel.

oracle/build_ref.sh compiles the reference's IsosurfaceApproximation.cu
(device code, nvcc default flags) into oracle/_ref/ref_approx.cubin;
oracle/refgpu.py runs its calculate_approximation_g on this GPU with the host
steps of approximate_isosurfaces_h (IsosurfaceApproximation.cu:159-208):
cells set to all-ones bytes, launches of 32,768 blocks at increasing block
offsets, and the stable compaction of the crossing cells.

Bar: the crossing cells, in order, equal bit for bit between the reference's
kernel, the engine's drop-in entry and the engine's SURFACE_APPROX surfaces.
"""
import numpy as np
import pytest

import refgpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_cubin():
    if not refgpu.approx_available():
        pytest.skip("reference cubin (oracle/_ref/ref_approx.cubin) not built")


def check(vol, dims, isos):
    import isosim
    with isosim.Context(0) as ctx:
        pts, _ = ctx.surface_points(vol.ravel(), dims, isos, surface=isosim.SURFACE_APPROX)
    nonempty = 0
    for k, iso in enumerate(isos):
        ref = refgpu.approximation(vol.ravel(), dims, float(iso))
        got = isosim.approximate_isosurfaces_h(vol.ravel(), dims, float(iso))
        assert np.array_equal(got, ref), iso
        assert np.array_equal(pts[k].astype(np.int32), ref), iso
        nonempty += len(ref) > 0
    return nonempty


def test_blobs_64():
    """64^3 blobs, eight of the 32 isovalues."""
    import isosim.synth as synth
    vol, isos, _ = synth.config1()
    assert check(vol, (64, 64, 64), isos[::4]) == 8


def test_large_volume_several_launches():
    """256^3 blobs + noise: 65,536 blocks of 256 threads, so two launches at
    block offsets 0 and 32,768; three isovalues."""
    import isosim.synth as synth
    vol, isos, _ = synth.config3()
    assert check(vol, (256, 256, 256), isos[[16, 128, 240]]) == 3


def test_ragged_grid_and_ties():
    """A 37 x 23 x 41 grid with values on a coarse lattice, so that corners
    equal to the isovalue (neither above nor below) occur."""
    rng = np.random.default_rng(41)
    dims = (37, 23, 41)
    vol = (rng.integers(0, 5, size=dims) / np.float32(4)).astype(np.float32)
    assert check(vol, dims, np.array([0.25, 0.5, 0.625], np.float32)) == 3
