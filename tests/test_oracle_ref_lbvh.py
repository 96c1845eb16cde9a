"""The oracle's restatement of the reference's LBVH construction (the check
the GPU checker runs before it executes the reference's BVH kernels)."""
import numpy as np

import oracle


def test_morton_known_values():
    p = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5], [1.0, 1.0, 1.0], [2.0, -1.0, 0.25]], np.float32)
    c = oracle.ref_morton(p)
    assert c[0] == 0
    assert c[1] == 7 << 27                  # 512 on every axis: bit 9 -> bits 27..29
    assert c[2] == (1 << 30) - 1            # clamped to 1023 on every axis
    # x clamped to 1023, y to 0, z = 256 (bit 8 -> bit 24)
    assert c[3] == (0x09249249 << 2) | (1 << 24)


def test_distinct_codes_balanced():
    l, r, depth = oracle.ref_lbvh(np.arange(8, dtype=np.uint32))
    assert depth == 3
    # root splits 0..3 | 4..7
    assert (l[0], r[0]) == (3, 4)


def test_duplicate_run_is_a_chain():
    """Equal codes take the reference's duplicate branch: a chain."""
    l, r, depth = oracle.ref_lbvh(np.full(6, 5, np.uint32))
    assert depth == 5
    assert list(l) == [-1, -2, -3, -4, -5]       # leaf i on the left of node i
    assert list(r) == [1, 2, 3, 4, -6]


def test_random_codes_valid_trees():
    rng = np.random.default_rng(1)
    for n in (2, 3, 17, 1000, 20000):
        c = np.sort(rng.integers(0, 1 << 30, n).astype(np.uint32))
        _, _, depth = oracle.ref_lbvh(c)
        assert 0 < depth <= 60, (n, depth)
    c = np.sort(rng.integers(0, 64, 5000).astype(np.uint32))   # long duplicate runs
    _, _, depth = oracle.ref_lbvh(c)
    assert depth > 0
