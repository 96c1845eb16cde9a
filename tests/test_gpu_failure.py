"""Failure detection without a GPU fault: the kernels' device-side waits are
bounded by time and report an error status instead of hanging.

iso_probe_wait_timeout runs the bounded barrier wait of the tensor-core
distance kernel on a barrier that nothing arrives at (a flag nothing sets):
the wait gives up after its limit, the kernel returns normally, the host reads
the status, and the context keeps working."""
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_wait_gives_up_and_the_context_stays_usable():
    import isosim
    with isosim.Context(0) as ctx:
        t0 = time.perf_counter()
        assert ctx.probe_wait_timeout(arrive=False, limit_ns=20_000_000)   # 20 ms
        assert time.perf_counter() - t0 < 2.0
        assert not ctx.probe_wait_timeout(arrive=True, limit_ns=20_000_000)
        # the same context afterwards: a tensor-core distance field, exact
        rng = np.random.default_rng(3)
        pts = rng.uniform(0.1, 0.9, (3000, 3)).astype(np.float32)
        dims = (24, 20, 28)
        got = ctx.distance_field(pts, dims, method=isosim.DF_TC)
        assert np.array_equal(got, oracle.distance_field_f32(pts, dims))


def test_probe_rejects_bad_limits():
    import isosim
    with isosim.Context(0) as ctx:
        with pytest.raises(isosim.IsoError):
            ctx.probe_wait_timeout(arrive=False, limit_ns=-1)
        with pytest.raises(isosim.IsoError):
            ctx.probe_wait_timeout(arrive=False, limit_ns=20_000_000_000)
