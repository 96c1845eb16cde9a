"""The serving loop: requests of different shapes, isovalue counts and bins
run concurrently under an HBM budget, and each result equals the result of
the same request run alone (bit for bit: every request reads only its own
buffers)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def requests():
    import isosim
    import isosim.synth as synth
    out = []
    shapes = [(24, 24, 24), (32, 28, 20), (40, 32, 28), (20, 20, 20), (36, 36, 36), (28, 24, 32)]
    for k, dims in enumerate(shapes):
        if k % 2 == 0:
            vol = synth.gaussian_blobs(dims, 5, 100 + k, sigma=(2.0, 6.0))
        else:
            vol = synth.power_law_field(dims, 3.0, 100 + k)
        n = [8, 16, 12, 24, 10, 20][k]
        isos = synth.inside_isovalues(vol, n)
        surface = isosim.SURFACE_APPROX if k == 3 else isosim.SURFACE_MC
        out.append((vol.ravel(), dims, isos, surface, [32, 64, 128, 16, 256, 64][k]))
    return out


def test_results_same_alone_and_in_the_mix():
    import isosim
    reqs = requests()
    with isosim.Context(0) as ctx:
        alone = [ctx.ism(v, d, i, surface=s, bins=b)[:2] for v, d, i, s, b in reqs]
    with isosim.Server(0, slots=3, budget_bytes=2 << 30) as srv:
        tickets = [srv.submit(v, d, i, surface=s, bins=b) for v, d, i, s, b in reqs * 3]
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for k, (ism, ids, res) in enumerate(results):
        want_ism, want_ids = alone[k % len(reqs)]
        assert res.status == 0
        assert np.array_equal(ids, want_ids)
        assert np.array_equal(ism, want_ism)
    assert st.completed == len(tickets) and st.failed == 0
    assert st.p50_ms > 0 and st.p99_ms >= st.p50_ms
    assert st.peak_device_bytes <= 2 << 30


def test_tight_budget_serialises_but_completes():
    import isosim
    reqs = requests()
    with isosim.Context(0) as ctx:
        alone = [ctx.ism(v, d, i, surface=s, bins=b)[0] for v, d, i, s, b in reqs]
    # room for about one request at a time
    with isosim.Server(0, slots=4, budget_bytes=96 << 20) as srv:
        tickets = [srv.submit(v, d, i, surface=s, bins=b) for v, d, i, s, b in reqs]
        for k, t in enumerate(tickets):
            ism, _, _ = srv.wait(t)
            assert np.array_equal(ism, alone[k])
        assert srv.stats().peak_device_bytes <= 96 << 20


def test_request_over_budget_fails_cleanly():
    import isosim
    import isosim.synth as synth
    vol = synth.gaussian_blobs((48, 48, 48), 5, 7, sigma=(3.0, 8.0))
    with isosim.Server(0, slots=2, budget_bytes=24 << 20) as srv:
        t = srv.submit(vol.ravel(), (48, 48, 48), synth.inside_isovalues(vol, 32), bins=64)
        with pytest.raises(isosim.IsoError) as e:
            srv.wait(t)
        assert e.value.code == isosim.ISO_ERR_NOMEM
        # the server keeps serving
        small = synth.gaussian_blobs((16, 16, 16), 3, 8, sigma=(2.0, 4.0))
        ism, ids, res = srv.wait(srv.submit(small.ravel(), (16, 16, 16), synth.inside_isovalues(small, 4), bins=16))
        assert res.status == 0 and len(ids) > 0


def test_waiters_do_not_hold_memory_the_earliest_needs():
    """Workers that finished large requests keep their arenas; when a second
    wave of large requests waits under a budget that fits one at a time, the
    waiters must release their arenas so the earliest one can run."""
    import isosim
    import isosim.synth as synth
    dims = (48, 48, 48)
    vol = synth.gaussian_blobs(dims, 6, 21, sigma=(3.0, 9.0))
    isos = synth.inside_isovalues(vol, 24)
    with isosim.Context(0) as ctx:
        want = ctx.ism(vol.ravel(), dims, isos, bins=64)[0]
    with isosim.Server(0, slots=3, budget_bytes=100 << 20) as srv:
        for wave in range(2):
            tickets = [srv.submit(vol.ravel(), dims, isos, bins=64) for _ in range(3)]
            for t in tickets:
                ism, _, _ = srv.wait(t)
                assert np.array_equal(ism, want)
        assert srv.stats().peak_device_bytes <= 100 << 20


def test_shortest_first_policy():
    """Shortest-first serving: the same results as alone (also on the
    high-priority stream), and small requests queued behind a big one are
    served before it unless the big one has waited longer than the bound."""
    import isosim
    import isosim.synth as synth
    reqs = requests()
    with isosim.Context(0) as ctx:
        alone = [ctx.ism(v, d, i, surface=s, bins=b)[:2] for v, d, i, s, b in reqs]
    big_vol = synth.gaussian_blobs((96, 96, 96), 6, 7, sigma=(6.0, 18.0))
    big_iso = synth.inside_isovalues(big_vol, 96)
    with isosim.Server(0, slots=1, budget_bytes=8 << 30) as srv:
        srv.set_policy(isosim.SERVE_SHORTEST_FIRST, 60000.0)
        first = srv.submit(big_vol.ravel(), (96, 96, 96), big_iso, bins=256)  # occupies the one worker
        queued_big = srv.submit(big_vol.ravel(), (96, 96, 96), big_iso, bins=256)
        small = [srv.submit(v, d, i, surface=s, bins=b) for v, d, i, s, b in reqs]
        res_small = [srv.wait(t) for t in small]
        _, _, r_big = srv.wait(queued_big)
        srv.wait(first)
    for k, (ism, ids, res) in enumerate(res_small):
        assert np.array_equal(ids, alone[k][1]) and np.array_equal(ism, alone[k][0])
        start = res.queue_ms
        assert start < r_big.queue_ms, k  # every small one started before the queued big one
    with isosim.Server(0, slots=3, budget_bytes=2 << 30) as srv:
        srv.set_policy(isosim.SERVE_SHORTEST_FIRST, 0.0)  # bound 0: the oldest always goes first
        tickets = [srv.submit(v, d, i, surface=s, bins=b) for v, d, i, s, b in reqs * 2]
        for k, t in enumerate(tickets):
            ism, ids, _ = srv.wait(t)
            assert np.array_equal(ism, alone[k % len(reqs)][0])


def test_reference_mi_mode_through_the_server():
    """The server's workers in the reference's FP32 MI mode: every request's
    map equals a context's map in that mode bit for bit; the setting is
    refused while requests are queued or running."""
    import isosim
    reqs = requests()
    with isosim.Context(0) as ctx:
        ctx.set_mi_mode(isosim.MI_REF32)
        alone = [ctx.ism(v, d, i, surface=s, bins=b)[:2] for v, d, i, s, b in reqs]
    with isosim.Server(0, slots=2, budget_bytes=4 << 30) as srv:
        srv.set_mi_mode(isosim.MI_REF32)
        tickets = [srv.submit(v, d, i, surface=s, bins=b) for v, d, i, s, b in reqs]
        with pytest.raises(isosim.IsoError):
            srv.set_mi_mode(isosim.MI_FP64)   # requests are queued or running
        for k, t in enumerate(tickets):
            ism, ids, _ = srv.wait(t)
            assert np.array_equal(ids, alone[k][1]) and np.array_equal(ism, alone[k][0]), k
        srv.set_mi_mode(isosim.MI_FP64)       # idle again
