"""CPU check of the histogram kernels' fixed-point bucket arithmetic.

The kernels bucket a value v of a pair with interval minimum mn and step
step = RN((mx - mn) / bins) as s = RN(RN(v - mn) * RN(1/step) + 1536) (one
fused multiply-add) and read the bucket from the bits of s; a value whose s
is an exact integer (other than 0) is re-bucketed by IEEE division.  This test
emulates that arithmetic bit for bit in integers (the exact product of the two
float32 significands, one round-to-nearest-even onto the 2^-13 grid of s) and
checks it against the reference's rule int(RN(RN(v - mn) / step)), clamped to
[0, bins - 1], for every value the fast path keeps.
"""
import numpy as np
import pytest

BASE = np.float32(1536.0)
BASE_BITS = 0x44C00000


def reference_bucket(v, mn, step, bins):
    d = (v - mn).astype(np.float32)
    q = (d / step).astype(np.float32)
    b = np.trunc(q).astype(np.int64)
    return np.clip(b, 0, bins - 1)


def _significand(x):
    """float32 -> (integer significand, exponent) with x = m * 2^e exactly."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.int64)
    ef = (b >> 23) & 0xFF
    m = np.where(ef == 0, b & 0x7FFFFF, (b & 0x7FFFFF) | 0x800000)
    e = np.where(ef == 0, -149, ef - 150)
    return m, e


def fixed_point_bucket(v, mn, step, bins):
    """Returns (bucket, ambiguous) as the kernels compute them."""
    r = np.float32(1.0) / np.float32(step)           # RN(1/step)
    d = (v - mn).astype(np.float32)                   # RN(v - mn), >= 0 here
    md, ed = _significand(d)
    mr, er = _significand(np.full_like(d, r))
    prod = md * mr                                    # < 2^48, exact
    sh = ed + er + 13                                 # d*r*2^13 = prod * 2^sh
    n = np.zeros_like(prod)
    up = sh >= 0
    n[up] = prod[up] << sh[up]
    k = np.clip(-sh, 1, 62)
    dn = (~up) & (-sh <= 62)
    q = prod >> k
    rem = prod & ((np.int64(1) << k) - 1)
    half = np.int64(1) << (k - 1)
    rnd = (rem > half) | ((rem == half) & ((q & 1) == 1))
    n[dn] = (q + rnd)[dn]                             # round half to even
    # s = 1536 + n * 2^-13 while n < 2^22 (q' < 512), so bits(s) = bits(1536) + n
    assert n.max(initial=0) < (1 << 22)
    u = BASE_BITS + n
    kb = BASE_BITS >> 13
    bucket = np.minimum(u >> 13, kb + bins - 1) - kb
    ambiguous = ((u & 0x1FFF) == 0) & (u != BASE_BITS)
    return bucket, ambiguous


def floor_bucket(v, mn, step, bins):
    """The kernels' bucket: RD(RN(v - mn) * RN(1/step) + 2^23) - 2^23 = the
    floor of the exact product, clamped to bins - 1 (exact integer emulation)."""
    r = np.float32(1.0) / np.float32(step)
    d = (v - mn).astype(np.float32)
    md, ed = _significand(d)
    mr, er = _significand(np.full_like(d, r))
    prod = md * mr
    sh = ed + er
    fl = np.zeros_like(prod)
    up = sh >= 0
    fl[up] = prod[up] << sh[up]
    k = np.clip(-sh, 0, 62)
    dn = (~up) & (-sh <= 62)
    fl[dn] = (prod >> k)[dn]
    return np.minimum(fl, bins - 1)


def intervals(rng, count):
    out = []
    for _ in range(count):
        kind = rng.integers(4)
        if kind == 0:
            mn, mx = 0.0, rng.uniform(1e-3, 2.0)
        elif kind == 1:
            mn = rng.uniform(1e-6, 0.05)
            mx = mn + rng.uniform(1e-4, 1.0)
        elif kind == 2:
            mn = rng.uniform(-5, 5)
            mx = mn + 10.0 ** rng.uniform(-4, 3)
        else:
            mn = 10.0 ** rng.uniform(-30, -20)
            mx = mn + 10.0 ** rng.uniform(-25, -18)
        out.append((np.float32(mn), np.float32(mx)))
    return out


@pytest.mark.parametrize("bins", [2, 16, 100, 128, 255, 256])
def test_fast_path_agrees_with_division(bins):
    rng = np.random.default_rng(bins)
    kept = flagged = 0
    for mn, mx in intervals(rng, 40):
        step = np.float32((mx - mn) / np.float32(bins))
        if not (np.isfinite(step) and step >= np.finfo(np.float32).tiny):
            continue
        k = np.arange(bins + 1, dtype=np.float32)
        edges = (mn + k * step).astype(np.float32)
        edges = edges[(edges >= mn) & (edges <= mx)]
        vals = np.concatenate([
            rng.uniform(mn, mx, 20000).astype(np.float32),
            edges,
            np.nextafter(edges, np.float32(np.inf)),
            np.nextafter(edges, np.float32(-np.inf)),
            np.array([mn, mx], np.float32),
        ]).astype(np.float32)
        vals = vals[(vals >= mn) & (vals <= mx)]
        ref = reference_bucket(vals, mn, step, bins)
        fx, amb = fixed_point_bucket(vals, mn, step, bins)
        ok = ~amb
        assert np.array_equal(fx[ok], ref[ok]), (mn, mx, bins)
        # the bucket the kernels count (floor of the exact product) agrees too
        assert np.array_equal(floor_bucket(vals, mn, step, bins)[ok], ref[ok]), (mn, mx, bins)
        kept += int(ok.sum())
        flagged += int(amb.sum())
        # v == mn (q = 0) stays on the fast path
        f0, a0 = fixed_point_bucket(np.array([mn], np.float32), mn, step, bins)
        assert f0[0] == 0 and not a0[0]
    assert kept > 100000
    # the exact division is rare: about 2^-13 of random values plus the edges
    assert flagged < 0.05 * kept


def test_every_value_stays_inside_the_histogram():
    """Values at and beyond the interval's ends still give a bucket in
    [0, bins - 1] (the kernels clamp the bin as a whole as well)."""
    mn, mx, bins = np.float32(0.25), np.float32(3.0), 256
    step = np.float32((mx - mn) / np.float32(bins))
    v = np.array([mx, np.nextafter(mx, np.float32(9)), mx * 1.001], np.float32)
    fx, _ = fixed_point_bucket(v, mn, step, bins)
    assert fx.min() >= 0 and fx.max() <= bins - 1


def test_lowest_set_bit_form_of_the_ambiguity_test():
    """The kernels test 'w is a nonzero multiple of 2^13' (u = bits(1536) | w)
    as 'the lowest set bit of u lies in bits 13..21' so that eight values
    combine with one OR; exhaustive over every u of the fixed-point range."""
    u = (BASE_BITS + np.arange(1 << 22, dtype=np.int64)).astype(np.uint32)
    direct = ((u & 0x1FFF) == 0) & (u != BASE_BITS)
    low = u & (np.uint32(0) - u)
    assert np.array_equal((low & np.uint32(0x3FE000)) != 0, direct)


def test_multiply_high_forms():
    """x >> 13 == umulhi(x, 2^19) and x >> 1 == umulhi(x, 2^31); the counted
    half of a word wraps exactly when old * (65536 - odd * 65535) >= 0xFFFF0000."""
    rng = np.random.default_rng(4)
    x = rng.integers(0, 1 << 32, 100000, dtype=np.uint64)
    assert np.array_equal((x * (1 << 19)) >> 32, x >> 13)
    assert np.array_equal((x * (1 << 31)) >> 32, x >> 1)
    old = np.concatenate([x, [0xFFFF, 0xFFFF0000, 0x1234FFFF, 0xFFFF1234, 0xFFFFFFFF, 0]]).astype(np.uint64)
    for odd in (0, 1):
        sh = 65536 - odd * 65535
        t = (old * sh) & 0xFFFFFFFF
        half = (old >> (16 * odd)) & 0xFFFF
        assert np.array_equal(t >= 0xFFFF0000, half == 0xFFFF)
