"""The allocation-free similarity map, called through the C ABI.

It serves callers that may not allocate GPU memory while they run (a fixed
memory budget committed up front, or a code path where the allocator must not
be entered).  Its output must match the regular entry point's on the same
fields and the FP64 oracle's, on consecutive calls that share its fixed
scratch array.  This file is collected last so a failure here cannot hide
other results."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-6  # the tolerance the similarity-map parity tests use


def _noalloc_fn():
    import isosim
    fn = isosim.lib.iso_similarity_map_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p]
    return fn


def _fields(m, n, seed):
    rng = np.random.default_rng(seed)
    base = rng.uniform(0, 1, n)
    return np.stack([np.abs(base * (1 + 0.3 * k) + 0.2 * rng.standard_normal(n)) for k in range(m)]).astype(np.float32)


def _concentrated(m, n, seed):
    """Fields whose values crowd into one bin: many 16-bit counter wraps."""
    rng = np.random.default_rng(seed)
    f = np.zeros((m, n), np.float32)
    f[:, :: 97] = rng.uniform(0, 1, (m, len(range(0, n, 97)))).astype(np.float32)
    f[1:] += np.float32(1e-3) * np.arange(1, m, dtype=np.float32)[:, None]
    return f


def _call(fn, host, bins, stream):
    import torch
    import isosim
    m, n = host.shape
    stride = (n + 63) // 64 * 64
    dev = torch.zeros((m, stride), dtype=torch.float32, device="cuda")
    dev[:, :n] = torch.from_numpy(host).cuda()
    out = torch.full((m, m), -1.0, dtype=torch.float32, device="cuda")
    rc = fn(C.c_void_p(dev.data_ptr()), m, n, stride, bins, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert rc == 0, isosim.last_error()
    return out.cpu().numpy()


@pytest.mark.parametrize("cases", [
    # fused-kernel lengths at 256 and 128 bins
    [(12, 300001, 256, "spread"), (7, 70003, 128, "spread")],
    # a length above 2,097,152 values, where the regular entry switches to its
    # segment-major kernels; then few bins over crowded fields (wraps)
    [(5, 2500003, 256, "spread"), (3, 1000003, 2, "crowded"), (3, 1000003, 6, "crowded"),
     (4, 400001, 30, "crowded")],
])
def test_noalloc_matches_regular_entry_and_oracle(cases):
    """Consecutive calls sharing the fixed scratch array, each checked against
    the regular entry point and the FP64 oracle."""
    import torch
    import isosim
    import oracle
    fn = _noalloc_fn()
    stream = torch.cuda.current_stream().cuda_stream
    with isosim.Context(0) as ctx:
        for call, (m, n, bins, kind) in enumerate(cases):
            host = _fields(m, n, seed=40 + call) if kind == "spread" else _concentrated(m, n, seed=50 + call)
            got = _call(fn, host, bins, stream)
            assert np.abs(got - ctx.similarity_map(host, bins)).max() < TOL, (call, bins)
            assert np.abs(got - oracle.similarity_map(host, bins, mode=0)).max() < TOL, (call, bins)


def test_noalloc_rejects_sizes_beyond_its_limits():
    import torch
    import isosim
    fn = _noalloc_fn()
    dev = torch.zeros(64, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(C.c_void_p(dev.data_ptr()), 257, 16, 16, 64, C.c_void_p(out.data_ptr()), s)
    assert rc == isosim.ISO_ERR_CAPACITY and "limit" in isosim.last_error()
    rc = fn(C.c_void_p(dev.data_ptr()), 2, 16777217, 16777220, 64, C.c_void_p(out.data_ptr()), s)
    assert rc == isosim.ISO_ERR_CAPACITY and "limit" in isosim.last_error()
