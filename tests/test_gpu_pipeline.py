"""The whole-volume pipeline against the oracle chain, plus size-independent
properties at the benchmark sizes."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-6


def oracle_chain(vol, dims, isos, bins, surface, frame, ds=1):
    fields, ids = [], []
    for k, iso in enumerate(isos):
        if surface == 0:
            pts, _, _ = oracle.marching_cubes(vol, dims, float(iso), frame=frame)
        else:
            pts = oracle.approximation(vol, dims, float(iso)).astype(np.float32)
        if len(pts) == 0:
            continue
        fields.append(oracle.distance_field_f32(oracle.normalize_points(pts, dims), dims, ds))
        ids.append(k)
    return oracle.similarity_map(np.stack(fields), bins, mode=0), np.array(ids, np.int32), np.stack(fields)


@pytest.mark.parametrize("surface,frame", [(0, 0), (0, 1), (1, 0)])
def test_small_volume_matches_oracle(ctx, surface, frame):
    import isosim
    import isosim.synth as synth
    dims = (20, 18, 16)
    vol = synth.gaussian_blobs(dims, 4, 77, sigma=(2.0, 5.0))
    isos = np.concatenate([synth.inside_isovalues(vol, 7), [vol.max() + 1.0]]).astype(np.float32)
    for method in (isosim.DF_BRUTE, isosim.DF_LBVH):
        ism, ids, stats, _ = ctx.ism(vol.ravel(), dims, isos, surface=surface, frame=frame, df_method=method, bins=32)
        want, want_ids, _ = oracle_chain(vol, dims, isos, 32, surface, frame)
        assert np.array_equal(ids, want_ids)
        assert np.abs(ism - want).max() < TOL
        assert stats[len(isos) - 1].points == 0


def test_downscaled_pipeline(ctx):
    import isosim.synth as synth
    dims = (24, 24, 24)
    vol = synth.gaussian_blobs(dims, 3, 5, sigma=(3.0, 6.0))
    isos = synth.inside_isovalues(vol, 5)
    ism, ids, _, _ = ctx.ism(vol.ravel(), dims, isos, downscale=2, bins=16)
    want, want_ids, _ = oracle_chain(vol, dims, isos, 16, 0, 0, ds=2)
    assert np.array_equal(ids, want_ids)
    assert np.abs(ism - want).max() < TOL


def test_config1_properties_and_methods(ctx):
    """64^3, 32 isovalues, 128 bins: brute force and LBVH give the same ISM
    bit for bit; the ISM is symmetric with a unit diagonal; repeat runs are
    bitwise identical; representatives match the oracle's selection."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config1()
    a, ids, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, df_method=isosim.DF_LBVH, bins=bins)
    b, ids2, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, df_method=isosim.DF_BRUTE, bins=bins)
    c, _, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, df_method=isosim.DF_LBVH, bins=bins)
    assert np.array_equal(ids, ids2) and np.array_equal(a, b) and np.array_equal(a, c)
    assert np.array_equal(a, a.T)
    assert np.all(np.abs(np.diag(a) - 1.0) < 1e-6)
    assert np.all((a >= -1e-6) & (a <= 1 + 1e-6))
    reps = isosim.select_representatives(a, ids, isos, 16)
    assert reps == oracle.select_representatives(a, ids, isos, 16)


def test_device_resident_volume_matches_host(ctx):
    import torch
    import isosim.synth as synth
    vol, isos, bins = synth.config1(seed=1001)
    a, _, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos[:8], bins=bins)
    dv = torch.from_numpy(vol.ravel()).cuda()
    b, _, _, _ = ctx.ism(dv, (64, 64, 64), isos[:8], bins=bins)
    assert np.array_equal(a, b)


def test_isovalue_selection_and_range(ctx):
    import isosim.synth as synth
    vol, _, _ = synth.config1(seed=1002)
    lo, hi = ctx.real_range(vol.ravel(), -1e9, 1e9)
    assert (lo, hi) == oracle.real_range(vol, -1e9, 1e9)
    lo2, hi2 = ctx.real_range(vol.ravel(), 0.1, 0.9)
    assert (lo2, hi2) == oracle.real_range(vol, 0.1, 0.9)
    for uniform in (True, False):
        assert np.array_equal(ctx.isovalues(vol.ravel(), lo, hi, 32, uniform),
                              oracle.isovalues(vol, lo, hi, 32, uniform))


def test_lbvh_groups_give_the_same_fields():
    """Distance fields built over many small LBVH groups equal one large group."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config1(seed=1003)
    with isosim.Context(0) as a, isosim.Context(0) as b:
        b.set_lbvh_group_points(3000)
        ia, ida, _, _ = a.ism(vol.ravel(), (64, 64, 64), isos, bins=bins)
        ib, idb, _, _ = b.ism(vol.ravel(), (64, 64, 64), isos, bins=bins)
    assert np.array_equal(ida, idb) and np.array_equal(ia, ib)


@pytest.mark.parametrize("surface", [0, 1])
def test_config1_full_size_matches_oracle(ctx, surface):
    """The 64^3, 32-isovalue, 128-bin workload at full size: surfaces, distance
    fields (oracle through its exact k-d tree) and the FP64 similarity map."""
    from concurrent.futures import ThreadPoolExecutor
    import isosim.synth as synth
    vol, isos, bins = synth.config1()
    dims = (64, 64, 64)
    ism, ids, stats, _ = ctx.ism(vol.ravel(), dims, isos, surface=surface, bins=bins)

    def field(k):
        if surface == 0:
            pts, active, total = oracle.marching_cubes(vol, dims, float(isos[k]), frame=0)
            assert stats[k].active_voxels == active and stats[k].total_verts == total
        else:
            pts = oracle.approximation(vol, dims, float(isos[k])).astype(np.float32)
        assert stats[k].points == len(pts)
        return oracle.distance_field_kd(oracle.normalize_points(pts, dims), dims) if len(pts) else None

    with ThreadPoolExecutor(8) as ex:
        fields = list(ex.map(field, range(len(isos))))
    want_ids = np.array([k for k, f in enumerate(fields) if f is not None], np.int32)
    assert np.array_equal(ids, want_ids)
    want = oracle.similarity_map(np.stack([f for f in fields if f is not None]), bins, mode=0)
    assert np.abs(ism - want).max() < TOL
