"""CPU check of the histogram kernels' bracketed bucket arithmetic.

The kernels bucket a value v of a pair with interval minimum mn and step
step = RN((mx - mn) / bins) from d = RN(v - mn) and two widened reciprocals
of r = RN(1/step): rlo = RD(r * (1 - 2^-22)) and rhi = RU(r * (1 + 2^-22)).
Two packed fused multiply-adds give floor(d * rlo) and floor(d * rhi)
exactly; where they agree that floor is the bucket, otherwise (and for NaN)
the value is re-bucketed by IEEE division.  This test emulates that
arithmetic bit for bit in integers (exact products of float32 significands)
and checks it against the reference's rule int(RN(RN(v - mn) / step)),
clamped to [0, bins - 1], for every value the fast path keeps.
"""
import numpy as np
import pytest

LO = 1.0 - 2.0 ** -22
HI = 1.0 + 2.0 ** -22


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


def exact_floor(d, r, bins):
    """floor(d * r) of float32 d >= 0 and float32 r, exactly, clamped to bins - 1:
    what RD(d * r + 2^23) - 2^23 gives in one fused multiply-add."""
    md, ed = _significand(d)
    mr, er = _significand(np.full_like(d, r))
    prod = md * mr                                    # < 2^48, exact
    sh = ed + er
    fl = np.zeros_like(prod)
    up = sh >= 0
    fl[up] = prod[up] << sh[up]
    k = np.clip(-sh, 0, 62)
    dn = (~up) & (-sh <= 62)
    fl[dn] = (prod >> k)[dn]
    return np.minimum(fl, bins - 1)


def widened_reciprocals(step):
    """(RD(r * (1 - 2^-22)), RU(r * (1 + 2^-22))) with r = RN(1/step); both
    products are exact in float64 and then rounded once to float32."""
    r = np.float32(1.0) / np.float32(step)
    lo64, hi64 = float(r) * LO, float(r) * HI
    lo, hi = np.float32(lo64), np.float32(hi64)
    if float(lo) > lo64:
        lo = np.nextafter(lo, np.float32(-np.inf))
    if float(hi) < hi64:
        hi = np.nextafter(hi, np.float32(np.inf))
    return lo, hi


def bracket_bucket(v, mn, step, bins):
    """Returns (bucket, ambiguous) as the kernels compute them."""
    d = (v - mn).astype(np.float32)                   # RN(v - mn), >= 0 here
    rlo, rhi = widened_reciprocals(step)
    flo = exact_floor(d, rlo, bins + 2)
    fhi = exact_floor(d, rhi, bins + 2)
    return np.minimum(flo, bins - 1), flo != fhi


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
        fx, amb = bracket_bucket(vals, mn, step, bins)
        ok = ~amb
        assert np.array_equal(fx[ok], ref[ok]), (mn, mx, bins)
        kept += int(ok.sum())
        flagged += int(amb.sum())
        # v == mn (q = 0) stays on the fast path
        f0, a0 = bracket_bucket(np.array([mn], np.float32), mn, step, bins)
        assert f0[0] == 0 and not a0[0]
    assert kept > 100000
    # the exact division is rare: about 2^-21 * q of random values plus edges
    assert flagged < 0.05 * kept


def test_bracket_holds_at_every_quotient_boundary():
    """Values whose quotient lies within a few ulps of every integer k, for
    steps with awkward reciprocals: the floors bracket the reference's bucket
    (floor(d * rlo) <= bucket <= floor(d * rhi)) for every one of them."""
    rng = np.random.default_rng(11)
    for _ in range(200):
        bins = int(rng.choice([2, 7, 100, 224, 256]))
        mn = np.float32(rng.uniform(-3, 3))
        step = np.float32(10.0 ** rng.uniform(-6, 2))
        mx = np.float32(mn + np.float32(bins) * step)
        step = np.float32((mx - mn) / np.float32(bins))
        if not (np.isfinite(step) and step > 0):
            continue
        k = np.arange(1, bins, dtype=np.float64)
        v = (np.float64(mn) + k * np.float64(step)).astype(np.float32)
        around = [v]
        for _ in range(3):
            around.append(np.nextafter(around[-1], np.float32(np.inf)))
        w = v
        for _ in range(3):
            w = np.nextafter(w, np.float32(-np.inf))
            around.append(w)
        vals = np.concatenate(around)
        vals = vals[(vals >= mn) & (vals <= mx)]
        ref = reference_bucket(vals, mn, step, bins)
        d = (vals - mn).astype(np.float32)
        rlo, rhi = widened_reciprocals(step)
        flo = exact_floor(d, rlo, 1 << 20)
        fhi = exact_floor(d, rhi, 1 << 20)
        assert np.all(np.minimum(flo, bins - 1) <= ref) and np.all(ref <= np.minimum(fhi, bins - 1))


def test_every_value_stays_inside_the_histogram():
    """Values at and beyond the interval's ends still give a bucket in
    [0, bins - 1] (the kernels clamp the bin as a whole as well)."""
    mn, mx, bins = np.float32(0.25), np.float32(3.0), 256
    step = np.float32((mx - mn) / np.float32(bins))
    v = np.array([mx, np.nextafter(mx, np.float32(9)), mx * 1.001], np.float32)
    fx, _ = bracket_bucket(v, mn, step, bins)
    assert fx.min() >= 0 and fx.max() <= bins - 1


def test_wrap_test_form():
    """The counted half of a word wraps exactly when old * (inc ^ 0x10001)
    >= 0xFFFF0000 (low 32 bits of the product), inc = odd * 0xFFFF + 1 being
    the half's increment (1 or 65536)."""
    rng = np.random.default_rng(4)
    x = rng.integers(0, 1 << 32, 100000, dtype=np.uint64)
    old = np.concatenate([x, [0xFFFF, 0xFFFF0000, 0x1234FFFF, 0xFFFF1234, 0xFFFFFFFF, 0]]).astype(np.uint64)
    for odd in (0, 1):
        inc = odd * 0xFFFF + 1
        sh = inc ^ 0x10001
        assert sh == 65536 - odd * 65535
        t = (old * sh) & 0xFFFFFFFF
        half = (old >> (16 * odd)) & 0xFFFF
        assert np.array_equal(t >= 0xFFFF0000, half == 0xFFFF)
