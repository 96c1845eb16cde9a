"""The autotuner: the shapes it may choose give identical results; it applies
its choice, caches it and reads the cache back without trials."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_query_runs_give_identical_fields():
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config1(seed=1005)
    with isosim.Context(0) as ctx:
        ref, ids, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, bins=bins)
        f0 = [ctx.copy_field(r, np.zeros(64 ** 3, np.float32)) for r in range(len(ids))]
        for run in (8, 16, 32, 64):
            ctx.set_query_run(run)
            got, ids2, _, _ = ctx.ism(vol.ravel(), (64, 64, 64), isos, bins=bins)
            assert np.array_equal(ids, ids2) and np.array_equal(got, ref), run
            for r in range(len(ids)):
                assert np.array_equal(ctx.copy_field(r, np.zeros(64 ** 3, np.float32)), f0[r]), (run, r)


def test_autotune_applies_and_caches(tmp_path):
    import isosim
    import isosim.synth as synth
    vol, isos, _ = synth.config3(size=96, n=48)
    dims = (96, 96, 96)
    cache = str(tmp_path / "tune.txt")
    with isosim.Context(0) as ctx:
        ctx.set_hist_segment_values(65536)  # a poor start: the tuner must not keep a slower set
        before, ids, _, _ = ctx.ism(vol.ravel(), dims, isos, bins=256)
        t = ctx.autotune(vol.ravel(), dims, isos, bins=256, cache_path=cache)
        assert t.from_cache == 0 and t.trials > 0
        assert t.tuned_ms <= t.default_ms
        assert t.query_run in (0, 8, 16, 32, 64)
        after, ids2, _, _ = ctx.ism(vol.ravel(), dims, isos, bins=256)
        assert np.array_equal(ids, ids2) and np.array_equal(before, after)
    lines = open(cache).read().strip().splitlines()
    assert len(lines) == 1 and "96x96x96" in lines[0]
    with isosim.Context(0) as ctx:
        t2 = ctx.autotune(vol.ravel(), dims, isos, bins=256, cache_path=cache)
        assert t2.from_cache == 1 and t2.trials == 0
        assert (t2.hist_segment_values, t2.lbvh_group_points, t2.query_run) == \
            (t.hist_segment_values, t.lbvh_group_points, t.query_run)
        again, _, _, _ = ctx.ism(vol.ravel(), dims, isos, bins=256)
        assert np.array_equal(again, before)
