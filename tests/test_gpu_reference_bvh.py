"""The engine's distance fields against the reference's own LBVH kernels.

oracle/build_ref.sh compiles the reference's BVH.cu (device code, nvcc default
flags, so its own floating-point contraction) into oracle/_ref/ref_bvh.cubin;
oracle/refgpu.py runs its Morton, build, box and traversal kernels on this GPU
with the host steps of generateHierarchy_h (BVH.cu:815-875), after checking on
the CPU that the tree they build is a tree no deeper than the traversal's
stack holds.

Bar: every sample of the engine's fields (LBVH and brute force) equals the
oracle's canonical FP32 minimum, which uses the reference's compiled sum of
squares, fma(dz,dz, fma(dx,dx, dy*dy)).  The reference's own fields equal
them except where its traversal misses the exact minimum.  Its box distance
(distanceToBox_d, BVH.cu:440-506) leaves out the axes on which the sample is
inside the box and sums the other squares in another order than its point
distance, so a box can round one ulp above a point inside it.  When the best
distance so far is exactly that ulp above, the reference prunes the box and
keeps the larger value.  So the reference's value is never below the engine's
and differs in at most 1 sample in 100,000, by at most 2 ulp (measured: 1 of
262,144 samples at 64^3 and 1 of 2,097,152 at 128^3).
"""
import numpy as np
import pytest

import oracle
import refgpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_cubin():
    if not refgpu.bvh_available():
        pytest.skip("reference cubin (oracle/_ref/ref_bvh.cubin) not built")


def engine_field(pn, dims, ds=1, method=None):
    import isosim
    with isosim.Context(0) as ctx:
        return ctx.distance_field(pn, dims, downscale=ds, method=isosim.DF_LBVH if method is None else method)


def check_reference_field(ref, eng, what):
    """The reference's field against the exact one; returns the samples where
    the reference's pruning kept a larger value."""
    assert ref.shape == eng.shape
    assert np.all(ref >= eng), what
    bad = np.nonzero(ref != eng)[0]
    assert bad.size <= max(2, ref.size // 100000), (what, bad.size)
    two_ulp = np.nextafter(np.nextafter(eng[bad], np.float32(np.inf)), np.float32(np.inf))
    assert np.all(ref[bad] <= two_ulp), what
    return int(bad.size)


def surface_points(vol, dims, iso):
    pts, _, _ = oracle.marching_cubes(vol, dims, float(iso), frame=0)
    return oracle.normalize_points(pts, dims)


def test_blobs_64_all_methods():
    """64^3 blobs: eight of the 32 surfaces; engine LBVH = engine brute force
    = oracle, and the reference's LBVH against them."""
    import isosim
    import isosim.synth as synth
    vol, isos, _ = synth.config1()
    dims = (64, 64, 64)
    for k in range(0, 32, 4):
        pn = surface_points(vol, dims, isos[k])
        ref = refgpu.lbvh_distance_field(pn, dims)
        eng = engine_field(pn, dims)
        assert np.array_equal(eng, engine_field(pn, dims, method=isosim.DF_BRUTE)), k
        assert np.array_equal(eng, oracle.distance_field_f32(pn, dims)), k
        check_reference_field(ref, eng, k)


def test_downscaled_samples():
    """Downscale 2 and 4 (the reference's dfDownscale sample mapping)."""
    import isosim.synth as synth
    vol, isos, _ = synth.config1()
    dims = (64, 64, 64)
    pn = surface_points(vol, dims, isos[10])
    for ds in (2, 4):
        ref = refgpu.lbvh_distance_field(pn, dims, ds=ds)
        eng = engine_field(pn, dims, ds)
        assert np.array_equal(eng, oracle.distance_field_f32(pn, dims, ds)), ds
        check_reference_field(ref, eng, ds)


def test_power_law_128():
    """128^3 k^-3 field: a small, the largest (1.18 M points) and a medium
    surface, 2,097,152 samples each."""
    import isosim.synth as synth
    vol, isos, _ = synth.config2()
    dims = (128, 128, 128)
    for k in (90, 50, 10):
        pn = surface_points(vol, dims, isos[k])
        check_reference_field(refgpu.lbvh_distance_field(pn, dims), engine_field(pn, dims), k)


def test_duplicate_codes():
    """Points on a coarse lattice (runs of equal Morton codes and equal
    points), which take the reference's duplicate-code branch of the build."""
    rng = np.random.default_rng(8)
    dims = (48, 40, 56)
    pn = (rng.integers(0, 8, size=(5000, 3)) / np.float32(8)).astype(np.float32)
    codes = np.sort(oracle.ref_morton(pn))
    assert np.max(np.unique(codes, return_counts=True)[1]) > 3
    eng = engine_field(pn, dims)
    assert np.array_equal(eng, oracle.distance_field_f32(pn, dims))
    check_reference_field(refgpu.lbvh_distance_field(pn, dims), eng, "lattice")
