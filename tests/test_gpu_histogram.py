"""Joint histograms and NMI on the GPU against the oracle and the reference's
golden vectors.  Bin counts are bit-exact; the FP64 NMI matches the oracle's
FP64 NMI to float rounding.  The reference-named entry returns the
reference's own FP32 MI as the reference's kernel computes it on the device
(bit for bit: test_gpu_reference_kernel.py); against the same function run on
the host (the golden vectors, glibc logf and no multiply-add contraction) it
agrees within TOL_REF_HOST."""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_F64 = 1e-6       # FP64 NMI rounded to float, different summation order
TOL_REF_HOST = 1e-5  # device vs host evaluation of the reference's FP32 MI


def fields_like_df(m, n, seed):
    rng = np.random.default_rng(seed)
    base = rng.uniform(0, 1, n)
    return np.stack([np.abs(base * (1 + 0.25 * k) + 0.15 * rng.standard_normal(n)) for k in range(m)]).astype(np.float32)


def test_golden_small_reference_named_entry():
    import isosim
    g = np.load(os.path.join(GOLDEN, "simmap_small.npz"))
    fields, bins = g["fields"], int(g["bins"])
    mins = [oracle.field_interval(f)[0] for f in fields]
    maxs = [oracle.field_interval(f)[1] for f in fields]
    sim, cols, rows = isosim.calculate_histogram_h(list(fields), mins, maxs, bins)
    assert np.array_equal(cols, g["cols"])
    assert np.array_equal(rows, g["rows"])
    assert np.abs(sim - g["sim"]).max() < TOL_REF_HOST


@pytest.mark.parametrize("m,n,bins", [(6, 300001, 256), (9, 70001, 128), (3, 4097, 32), (2, 5, 16),
                                      (4, 50001, 224), (4, 50001, 226), (3, 20001, 100), (3, 9999, 62)])
def test_joint_histograms_bit_exact(ctx, m, n, bins):
    f = fields_like_df(m, n, seed=m * 7 + bins)
    ism, joint = ctx.similarity_map(f, bins, joint=True)
    for i in range(m):
        for j in range(m):
            want, _, _ = oracle.pair_histogram(f[i], f[j], bins)
            assert np.array_equal(joint[i, j], want), (i, j)
    want = oracle.similarity_map(f, bins, mode=0)
    assert np.abs(ism - want).max() < TOL_F64
    assert np.array_equal(ism, ism.T)


def test_ref32_mode_against_fp32_restatement():
    """ISO_MI_REF32 against the oracle's FP32 restatement (the host evaluation
    of the reference's function), and FP64 against FP64."""
    import isosim
    f = fields_like_df(5, 200003, seed=3)
    with isosim.Context(0) as c:
        ism64 = c.similarity_map(f, 128)
        c.set_mi_mode(isosim.MI_REF32)
        ism32 = c.similarity_map(f, 128)
    assert np.abs(ism32 - oracle.similarity_map(f, 128, mode=1)).max() < TOL_REF_HOST
    assert np.abs(ism64 - oracle.similarity_map(f, 128, mode=0)).max() < TOL_F64
    assert np.array_equal(ism64, ism64.T)


def test_constant_and_degenerate_fields(ctx):
    n = 10000
    f = np.stack([np.full(n, 0.25, np.float32), np.zeros(n, np.float32),
                  np.linspace(0, 1, n).astype(np.float32)])
    ism, joint = ctx.similarity_map(f, 64, joint=True)
    for i in range(3):
        for j in range(3):
            want, _, _ = oracle.pair_histogram(f[i], f[j], 64)
            assert np.array_equal(joint[i, j], want)
    want = oracle.similarity_map(f, 64, mode=0)
    assert np.abs(ism - want).max() < TOL_F64


def test_cross_map_and_multi_entry(ctx):
    import isosim
    a = fields_like_df(4, 50021, seed=11)
    b = fields_like_df(4, 50021, seed=12) * 1.5
    cm = ctx.cross_map(a, b, 64)
    for i in range(4):
        for j in range(4):
            lo_i, hi_i = oracle.field_interval(a[i])
            lo_j, hi_j = oracle.field_interval(b[j])
            joint, _, _ = oracle.pair_histogram(a[i], b[j], 64, (lo_i, hi_i), (lo_j, hi_j))
            assert abs(cm[i, j] - oracle.mi_f64(joint, a.shape[1])) < TOL_F64
    fields = list(a) + list(b)
    mins = [oracle.field_interval(x)[0] for x in fields]
    maxs = [oracle.field_interval(x)[1] for x in fields]
    sim, cols, rows = isosim.calculate_histogram_h(fields, mins, maxs, 64, multi=True)
    for i in range(4):
        for j in range(4):
            joint, cs, rs = oracle.pair_histogram(a[i], b[j], 64, (mins[i], maxs[i]), (mins[4 + j], maxs[4 + j]))
            assert np.array_equal(cols[i, j], cs) and np.array_equal(rows[i, j], rs)
            assert abs(sim[i, j] - oracle.mi_f32(joint, cs, rs, a.shape[1])) < TOL_REF_HOST


def test_deterministic(ctx):
    f = fields_like_df(7, 123457, seed=21)
    a = ctx.similarity_map(f, 256)
    b = ctx.similarity_map(f, 256)
    assert np.array_equal(a, b)


def test_bucket_boundaries_bit_exact(ctx):
    """Values exactly on bucket boundaries (min + k*step) and one ulp either
    side: the reciprocal fast path must hand every near-boundary value to the
    exact division."""
    bins = 256
    mn, mx = np.float32(0.0), np.float32(1.7)
    step = np.float32(mx - mn) / np.float32(bins)
    ks = np.arange(bins + 1, dtype=np.float32)
    on = (ks * step).astype(np.float32)
    vals = np.concatenate([on, np.nextafter(on, np.float32(-1)), np.nextafter(on, np.float32(9)),
                           [mn, mx]]).astype(np.float32)
    vals = np.clip(vals, mn, mx)
    rng = np.random.default_rng(2)
    n = 4 * len(vals)
    f1 = np.resize(vals, n).astype(np.float32)
    f2 = rng.permutation(f1).astype(np.float32)
    f = np.stack([f1, f2])
    _, joint = ctx.similarity_map(f, bins, joint=True)
    for i in range(2):
        for j in range(2):
            want, _, _ = oracle.pair_histogram(f[i], f[j], bins)
            assert np.array_equal(joint[i, j], want)


@pytest.mark.parametrize("bins", [2, 4, 256])
def test_counter_wraps(ctx, bins):
    """More than 65536 hits per bin.  With 256 bins the kernel packs two bins
    per 32-bit word; buckets 0 and 1 (one word) both get over 65536 hits, so
    the wrap corrections, including the carry out of a word, must restore the
    exact counts.  Smaller bin counts use one 32-bit counter per bin."""
    rng = np.random.default_rng(bins)
    n = 1_000_003
    if bins == 256:
        f = (rng.integers(0, 2, size=(3, n)) * (1.5 / 256)).astype(np.float32)
        f[:, 0] = 1.0  # interval [0, 1]: the two values land in buckets 0 and 1
    else:
        f = rng.integers(0, bins, size=(3, n)).astype(np.float32)
        f[:, 0] = 0
        f[:, 1] = bins - 1
    ism, joint = ctx.similarity_map(f, bins, joint=True)
    for i in range(3):
        for j in range(3):
            want, _, _ = oracle.pair_histogram(f[i], f[j], bins)
            assert np.array_equal(joint[i, j], want), (i, j)
    if bins == 256:
        assert joint[0, 1][:2, :2].min() > 65536
    assert np.abs(ism - oracle.similarity_map(f, bins, mode=0)).max() < TOL_F64


# ---- segment-major schedule (fields longer than one 262144-value segment) ----

SEG = 262144
DEFAULT_SEG = 2097152  # the engine's default segment length


@pytest.fixture
def seg_mode(ctx):
    """The session context with the segment-major schedule for fields longer
    than SEG values (off by default)."""
    ctx.set_hist_segment_values(SEG)
    yield
    ctx.set_hist_segment_values(DEFAULT_SEG)


@pytest.mark.usefixtures("seg_mode")
@pytest.mark.parametrize("n", [SEG + 1, 2 * SEG, 3 * SEG + 7])
def test_segmented_bit_exact(ctx, n):
    """Fields spanning several segments (a one-value last segment, an exact
    multiple, a ragged tail): every segment's counts land in the pair's
    histogram exactly once."""
    f = fields_like_df(4, n, seed=n % 97)
    ism, joint = ctx.similarity_map(f, 256, joint=True)
    for i in range(4):
        for j in range(4):
            want, _, _ = oracle.pair_histogram(f[i], f[j], 256)
            assert np.array_equal(joint[i, j], want), (i, j)
    assert np.abs(ism - oracle.similarity_map(f, 256, mode=0)).max() < TOL_F64
    assert np.array_equal(ism, ism.T)


@pytest.mark.usefixtures("seg_mode")
def test_segmented_wraps_in_both_halves(ctx):
    """Fields of two values that land in buckets 0 and 1 of 256 (one packed
    word): whole segments go to one bin (four 16-bit wraps per segment), to
    the even bin (low half, carries into the high half), the odd bin (high
    half, carry out of the word) and both halves of one word."""
    n = 4 * SEG + 3
    bins = 256
    rng = np.random.default_rng(5)
    lo_v, hi_v = np.float32(0.0), np.float32(1.5 / 256)
    half = np.where(rng.uniform(0, 1, n) < 0.5, lo_v, hi_v).astype(np.float32)
    f = np.stack([np.full(n, lo_v, np.float32), np.full(n, hi_v, np.float32), half,
                  np.where(half == lo_v, hi_v, lo_v).astype(np.float32)])
    f[:, 0] = 1.0   # every field spans [0, 1]: the two values are buckets 0 and 1
    ism, joint = ctx.similarity_map(f, bins, joint=True)
    for i in range(4):
        for j in range(4):
            want, _, _ = oracle.pair_histogram(f[i], f[j], bins)
            assert np.array_equal(joint[i, j], want), (i, j)
    assert np.abs(ism - oracle.similarity_map(f, bins, mode=0)).max() < TOL_F64


@pytest.mark.usefixtures("seg_mode")
def test_segmented_cross_map_and_sums(ctx):
    """Cross map on the session context (262,144-value segments) and the
    reference-named entry on the default one (fields just over the default
    segment length, so it runs segment-major too, with row and column sums)."""
    import isosim
    n = DEFAULT_SEG + 5
    a = fields_like_df(3, n, seed=31)
    b = fields_like_df(3, n, seed=32) * 1.5
    cm = ctx.cross_map(a, b, 256)
    fields = list(a) + list(b)
    mins = [oracle.field_interval(x)[0] for x in fields]
    maxs = [oracle.field_interval(x)[1] for x in fields]
    sim, cols, rows = isosim.calculate_histogram_h(fields, mins, maxs, 256, multi=True)
    for i in range(3):
        for j in range(3):
            joint, cs, rs = oracle.pair_histogram(a[i], b[j], 256, (mins[i], maxs[i]), (mins[3 + j], maxs[3 + j]))
            assert abs(cm[i, j] - oracle.mi_f64(joint, n)) < TOL_F64
            assert np.array_equal(cols[i, j], cs) and np.array_equal(rows[i, j], rs)
            assert abs(sim[i, j] - oracle.mi_f32(joint, cs, rs, n)) < TOL_REF_HOST


@pytest.mark.usefixtures("seg_mode")
def test_segmented_matches_fused(ctx):
    """The same pairs through the fused kernel (fields of one segment) and the
    segment-major kernels (the fields repeated three times, so every bin count
    triples): NMI is invariant under scaling all counts."""
    f = fields_like_df(5, SEG // 2, seed=77)
    fused = ctx.similarity_map(f, 256)
    seg = ctx.similarity_map(np.concatenate([f, f, f], axis=1), 256)
    assert np.abs(fused - seg).max() < TOL_F64


def test_schedules_agree(ctx):
    """The fused kernel (segmenting off) and the segment-major kernels at two
    segment lengths give identical histograms and ISMs."""
    f = fields_like_df(6, 3 * SEG + 11, seed=88)
    try:
        ctx.set_hist_segment_values(0)
        ism0, j0 = ctx.similarity_map(f, 256, joint=True)
        ctx.set_hist_segment_values(65536)
        ism1, j1 = ctx.similarity_map(f, 256, joint=True)
        ctx.set_hist_segment_values(SEG)
        ism2, j2 = ctx.similarity_map(f, 256, joint=True)
    finally:
        ctx.set_hist_segment_values(DEFAULT_SEG)
    assert np.array_equal(j0, j1) and np.array_equal(j0, j2)
    assert np.abs(ism0 - ism1).max() < TOL_F64 and np.abs(ism0 - ism2).max() < TOL_F64


def test_nan_values_take_bucket_zero(ctx):
    """NaN never enters a field interval (the comparisons in getInterval fail)
    and converts to bucket 0 in the reference's GPU kernel ((int)NaN is 0 on
    the device); the fast path hands NaN values to the division."""
    f = fields_like_df(3, 100003, seed=5)
    f[0, ::997] = np.nan
    f[2, 5::1231] = np.nan
    ism, joint = ctx.similarity_map(f, 64, joint=True)
    iv = [oracle.field_interval(x) for x in f]
    for i in range(3):
        for j in range(3):
            lo = min(iv[i][0], iv[j][0])
            a = np.where(np.isnan(f[i]), lo, f[i]).astype(np.float32)
            b = np.where(np.isnan(f[j]), lo, f[j]).astype(np.float32)
            want, _, _ = oracle.pair_histogram(a, b, 64, iv[i], iv[j])
            assert np.array_equal(joint[i, j], want), (i, j)


def test_reference_named_entry_256_bins():
    """Row and column sums of the reference-named entry at 256 bins (packed
    16-bit counters) against the oracle."""
    import isosim
    a = fields_like_df(3, 70001, seed=43)
    b = fields_like_df(3, 70001, seed=44) * 1.5
    fields = list(a) + list(b)
    mins = [oracle.field_interval(x)[0] for x in fields]
    maxs = [oracle.field_interval(x)[1] for x in fields]
    sim, cols, rows = isosim.calculate_histogram_h(fields, mins, maxs, 256, multi=True)
    for i in range(3):
        for j in range(3):
            joint_ij, cs, rs = oracle.pair_histogram(a[i], b[j], 256, (mins[i], maxs[i]), (mins[3 + j], maxs[3 + j]))
            assert np.array_equal(cols[i, j], cs) and np.array_equal(rows[i, j], rs)
            assert abs(sim[i, j] - oracle.mi_f32(joint_ij, cs, rs, a.shape[1])) < TOL_REF_HOST


def test_row_codes_bit_exact():
    """Segment-major histograms with precomputed row buckets: the same joint
    histograms and maps as without them -- symmetric runs (fields ordered by
    their maximum), cross maps (the coded field is sometimes the pair's second,
    so the shared histogram is transposed), a field whose minimum is far above
    the others' (many values near a bucket edge take the divisions) and the
    reference's FP32 MI over the dumped histograms."""
    import isosim
    n = 3 * SEG + 5
    f = fields_like_df(7, n, seed=71)
    f[2] += np.float32(0.05)          # a much larger minimum than the others
    f[5] *= np.float32(2.5)           # the largest maximum
    g = fields_like_df(7, n, seed=72)[::-1].copy() * np.float32(1.7)
    out = {}
    for codes in (0, 1):
        with isosim.Context(0) as c:
            c.set_hist_segment_values(SEG)
            c.set_hist_row_codes(codes)
            ism, joint = c.similarity_map(f, 256, joint=True)
            cm = c.cross_map(f, g, 256)
            c.set_mi_mode(isosim.MI_REF32)
            ism32 = c.similarity_map(f, 256)
            cm32 = c.cross_map(f, g, 256)
            out[codes] = (ism, joint, cm, ism32, cm32)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    for i in range(7):
        for j in range(7):
            want, _, _ = oracle.pair_histogram(f[i], f[j], 256)
            assert np.array_equal(out[1][1][i, j], want), (i, j)


@pytest.mark.parametrize("n", [300001, 2500003])
def test_values_above_caller_maxima_256_bins(n):
    """Caller-supplied maxima below the fields' largest values (the
    reference-named entry takes its intervals from its caller): those values
    count in the last bucket, as the reference clamps them, in the fused
    kernel (300,001 values) and the segment-major kernels (2,500,003); column
    and row sums bit-exact against the oracle, the map within the
    host-evaluation bound."""
    import isosim
    m = 4
    fields = list(fields_like_df(m, n, seed=n % 1000))
    mins, maxs = [], []
    for f in fields:
        lo, hi = oracle.field_interval(f)
        mins.append(float(lo))
        maxs.append(float(np.float32(hi - 0.2 * (hi - lo))))
    sim, cols, rows = isosim.calculate_histogram_h(fields, mins, maxs, 256)
    above = 0
    for i in range(m):
        for j in range(m):
            joint, cs, rs = oracle.pair_histogram(fields[i], fields[j], 256, (mins[i], maxs[i]), (mins[j], maxs[j]))
            assert np.array_equal(cols[i, j], cs) and np.array_equal(rows[i, j], rs), (i, j)
            assert abs(sim[i, j] - oracle.mi_f32(joint, cs, rs, n)) < TOL_REF_HOST
        above += int(np.count_nonzero(fields[i] > max(maxs)))
    assert above > 0


@pytest.mark.parametrize("n,bins", [(300001, 256), (2500003, 256), (70001, 128)])
def test_caller_intervals_wider_than_values(n, bins):
    """Caller-supplied intervals that contain every value, some wider than
    the field's own (lower minima, higher maxima): the 256- and 128-bin
    kernel instances then skip the fast path's bucket clamp.  Column and row
    sums bit-exact against the oracle with the same intervals, in the fused
    (300,001 and 70,001 values) and segment-major (2,500,003) kernels."""
    import isosim
    m = 4
    fields = list(fields_like_df(m, n, seed=n % 997 + bins))
    mins, maxs = [], []
    for k, f in enumerate(fields):
        lo, hi = oracle.field_interval(f)
        widen = 0.0 if k == 0 else 0.05 * k * (hi - lo)  # field 0 keeps its own interval
        mins.append(float(np.float32(lo - widen)))
        maxs.append(float(np.float32(hi + widen)))
    sim, cols, rows = isosim.calculate_histogram_h(fields, mins, maxs, bins)
    for i in range(m):
        for j in range(m):
            joint, cs, rs = oracle.pair_histogram(fields[i], fields[j], bins, (mins[i], maxs[i]), (mins[j], maxs[j]))
            assert np.array_equal(cols[i, j], cs) and np.array_equal(rows[i, j], rs), (i, j)
            assert abs(sim[i, j] - oracle.mi_f32(joint, cs, rs, n)) < TOL_REF_HOST


def test_values_below_caller_minimum_refused():
    """A caller-supplied minimum above one of its field's values is refused
    (the reference would index below its histogram)."""
    import isosim
    fields = list(fields_like_df(3, 50021, seed=5))
    mins = [float(np.float32(oracle.field_interval(f)[0] + 0.05)) for f in fields]
    maxs = [float(oracle.field_interval(f)[1]) for f in fields]
    with pytest.raises(isosim.IsoError, match="above its smallest value"):
        isosim.calculate_histogram_h(fields, mins, maxs, 256)
