"""The engine against the reference's own GPU histogram kernel.

oracle/build_ref.sh compiles the reference's JointHistogram.cu (device code,
nvcc default flags) into oracle/_ref/ref_histogram.cubin; oracle/refgpu.py
runs its calculate_histogram_g on this GPU as the reference's host driver
does.  That gives the reference's own output on the same fields: its joint
histograms, column and row sums, and its FP32 similarity map.

Bars:
  * joint histograms, column and row sums: bit-exact;
  * ISO_MI_REF32 (the reference-named entry's mode): every ISM entry equal to
    the reference's, bit for bit;
  * ISO_MI_FP64 (the engine's default): an accurate MI, which differs from
    the reference's FP32 evaluation by the reference's own rounding, up to
    GAP_F64 (the reference's map is itself asymmetric by about half that).
"""
import numpy as np
import pytest

import oracle  # noqa: F401  (tests/ puts oracle/ on the path)
import refgpu

pytestmark = pytest.mark.gpu
GAP_F64 = 2e-4   # |FP64 NMI - reference FP32 MI| on these workloads (measured up to 7e-5 at 64^3)


@pytest.fixture(scope="module", autouse=True)
def need_cubin():
    if not refgpu.available():
        pytest.skip("reference cubin (oracle/_ref/ref_histogram.cubin) not built")


def engine_fields(vol, dims, isos, bins, df_method):
    """ISMs in both MI modes and the distance fields behind them."""
    import isosim
    F = dims[0] * dims[1] * dims[2]
    with isosim.Context(0) as c:
        ism64, ids, _, _ = c.ism(vol.ravel(), dims, isos, df_method=df_method, bins=bins)
        fields = np.stack([c.copy_field(r, np.zeros(F, np.float32)) for r in range(len(ids))])
        c.set_mi_mode(isosim.MI_REF32)
        ism32, ids32, _, _ = c.ism(vol.ravel(), dims, isos, df_method=df_method, bins=bins)
    assert np.array_equal(ids, ids32)
    return fields, ism64, ism32


def check_against_reference(fields, ism64, ism32, bins):
    import isosim
    m = fields.shape[0]
    sim, joint, cols, rows = refgpu.similarity(fields, bins)
    # the engine's histograms are the reference's
    with isosim.Context(0) as c:
        _, ej = c.similarity_map(fields, bins, joint=True)
    assert np.array_equal(ej.reshape(m * m, bins, bins), joint)
    # the reference-named entry: sums and map bit for bit
    mins, maxs = fields.min(axis=1), fields.max(axis=1)
    hsim, hcols, hrows = isosim.calculate_histogram_h(list(fields), mins, maxs, bins)
    assert np.array_equal(hcols.reshape(m * m, bins), cols)
    assert np.array_equal(hrows.reshape(m * m, bins), rows)
    assert np.array_equal(hsim, sim)
    # the pipeline in both modes
    assert np.array_equal(ism32, sim)
    gap = float(np.abs(ism64 - sim).max())
    assert gap < GAP_F64, gap
    return gap


def test_config1_full_size():
    """64^3 blobs, 32 isovalues, brute-force FP32 distance fields, 128 bins:
    all 1024 ordered pairs against the reference's kernel."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config1()
    fields, ism64, ism32 = engine_fields(vol, (64, 64, 64), isos, bins, isosim.DF_BRUTE)
    assert fields.shape == (32, 64 ** 3)
    check_against_reference(fields, ism64, ism32, bins)


def test_config2_sixteen_fields():
    """128^3 k^-3 field, 16 of its 100 isovalues, 256 bins: fields of
    2,097,152 values, which the reference stages in three chunks."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config2()
    sel = isos[2::6][:16]
    fields, ism64, ism32 = engine_fields(vol, (128, 128, 128), sel, bins, isosim.DF_LBVH)
    assert fields.shape == (16, 128 ** 3)
    check_against_reference(fields, ism64, ism32, bins)


def test_segment_major_schedule():
    """Fields longer than the segment length at 256 bins go through the
    segment-major kernels (per-pair global histograms): REF32 over them."""
    import isosim
    rng = np.random.default_rng(17)
    n = 3000001
    base = rng.uniform(0, 1, n)
    f = np.stack([np.abs(base * (1 + 0.3 * k) + 0.1 * rng.standard_normal(n)) for k in range(4)]).astype(np.float32)
    sim, joint, _, _ = refgpu.similarity(f, 256)
    with isosim.Context(0) as c:
        c.set_mi_mode(isosim.MI_REF32)
        ism32, ej = c.similarity_map(f, 256, joint=True)
    assert np.array_equal(ej.reshape(16, 256, 256), joint)
    assert np.array_equal(ism32, sim)


def test_multi_mode_cross_map():
    """The multi mode of the reference-named entry (first m fields against the
    last m) against the reference's multi tasks (JointHistogram.cu:306-318)."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config1()
    fields, _, _ = engine_fields(vol, (64, 64, 64), isos[::4], bins, isosim.DF_LBVH)
    a, b = fields[:4], fields[4:8] * np.float32(1.25)
    both = np.concatenate([a, b])
    sim, _, cols, rows = refgpu.similarity(both, 256, multi=True)
    mins, maxs = both.min(axis=1), both.max(axis=1)
    hsim, hcols, hrows = isosim.calculate_histogram_h(list(both), mins, maxs, 256, multi=True)
    assert np.array_equal(hcols.reshape(16, 256), cols)
    assert np.array_equal(hrows.reshape(16, 256), rows)
    assert np.array_equal(hsim, sim)
    with isosim.Context(0) as c:
        c.set_mi_mode(isosim.MI_REF32)
        cm = c.cross_map(a, b, bins=256)
    assert np.array_equal(cm, sim)


@pytest.mark.parametrize("m", [96, 91])
def test_several_histogram_runs(m):
    """Maps whose histograms exceed one 2 GiB allocation at 256 bins, as the
    256^3 workload's do: 96 fields take two runs of 4,608 pairs, 91 fields
    (an odd pair count) two runs of 4,140 and a last run of one pair
    (calculateRunInfo, JointHistogram.cu:231-264); fields of 1,200,001 values
    in two chunks.  The reference-named entry's map and sums against the
    reference kernel's, bit for bit."""
    import isosim
    assert refgpu.run_info(m * m, m * m * 65536 * 4, m * m)[3] == (2 if m == 96 else 3)
    rng = np.random.default_rng(m)
    n = 1200001
    base = rng.uniform(0, 1, n)
    f = np.stack([np.abs(base * (1 + 0.02 * k) + 0.1 * rng.standard_normal(n)) for k in range(m)]).astype(np.float32)
    sim, joint, cols, rows = refgpu.similarity(f, 256)
    assert joint is None
    mins, maxs = f.min(axis=1), f.max(axis=1)
    hsim, hcols, hrows = isosim.calculate_histogram_h(list(f), mins, maxs, 256)
    assert np.array_equal(hcols.reshape(m * m, 256), cols)
    assert np.array_equal(hrows.reshape(m * m, 256), rows)
    assert np.array_equal(hsim, sim)


def test_config3_full_length_fields():
    """The 256^3 benchmark workload's own distance fields at full length
    (16,777,216 values: 16 chunks of 1,000,000 and a last one of 777,216),
    every fourth of its 256 fields (4,096 ordered pairs, one histogram run;
    the runs themselves are pinned above): the reference-named entry's map and
    sums against the reference kernel's, bit for bit, and the pipeline's
    ISO_MI_REF32 map on the same pairs."""
    import isosim
    import isosim.synth as synth
    vol, isos, bins = synth.config3()
    F = 256 ** 3
    with isosim.Context(0) as c:
        c.set_mi_mode(isosim.MI_REF32)
        ism32, ids, _, _ = c.ism(vol.ravel(), (256, 256, 256), isos, bins=bins)
        rows = list(range(0, len(ids), 4))
        fields = np.stack([c.copy_field(r, np.zeros(F, np.float32)) for r in rows])
    m = len(rows)
    sim, joint, cols, rws = refgpu.similarity(fields, bins)
    assert joint is not None and m == 64
    mins, maxs = fields.min(axis=1), fields.max(axis=1)
    hsim, hcols, hrows = isosim.calculate_histogram_h(list(fields), mins, maxs, bins)
    assert np.array_equal(hcols.reshape(m * m, bins), cols)
    assert np.array_equal(hrows.reshape(m * m, bins), rws)
    assert np.array_equal(hsim, sim)
    assert np.array_equal(ism32[np.ix_(rows, rows)], sim)


@pytest.mark.parametrize("bins", [2, 6, 30])
def test_few_bins(bins):
    """Bin counts whose histograms end inside a 32-bin staging step of the
    reference-order MI (4, 36 and 900 bins per pair): map and sums against the
    reference kernel's, bit for bit."""
    import isosim
    rng = np.random.default_rng(bins)
    n = 200003
    base = rng.uniform(0, 1, n)
    f = np.stack([np.abs(base * (1 + 0.2 * k) + 0.1 * rng.standard_normal(n)) for k in range(5)]).astype(np.float32)
    sim, joint, cols, rows = refgpu.similarity(f, bins)
    mins, maxs = f.min(axis=1), f.max(axis=1)
    hsim, hcols, hrows = isosim.calculate_histogram_h(list(f), mins, maxs, bins)
    assert np.array_equal(hcols.reshape(25, bins), cols)
    assert np.array_equal(hrows.reshape(25, bins), rows)
    assert np.array_equal(hsim, sim)
