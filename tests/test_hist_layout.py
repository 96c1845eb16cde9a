"""CPU model of the histogram kernels' padded shared-memory layout.

A shared histogram row is padded so that the same column of neighbouring rows
falls in different banks.  Packed 16-bit counters: counter index
row * (bins + 2 * PAD) + col, word index / 2, PAD pad words per row (3).
32-bit counters: row * (bins + 1) + col.  The segment-major kernel maps a
shared counter index and a shared word back to the unpadded global histogram
(row * bins + col); this test checks those maps over a range of bin counts,
and the bank spread the padding buys for voxels that share a column bin."""
import numpy as np
import pytest

PAD = 3


def packed_index(r, c, bins):
    return r * (bins + 2 * PAD) + c


@pytest.mark.parametrize("bins", [2, 4, 16, 62, 100, 226, 254, 256])
def test_packed_index_maps_back(bins):
    r, c = np.meshgrid(np.arange(bins), np.arange(bins), indexing="ij")
    idx = packed_index(r, c, bins)
    rs = bins + 2 * PAD
    # wrap corrections: shared counter index -> global index, same parity
    g = idx - 2 * PAD * (idx // rs)
    assert np.array_equal(g, r * bins + c)
    assert np.array_equal(g & 1, idx & 1)
    # flush: every word holding counters maps to the global index of its low counter
    w = idx >> 1
    wps = bins // 2 + PAD
    low = 2 * (w - PAD * (w // wps))
    assert np.array_equal(low, (r * bins + c) & ~1)
    # the pad words (word columns bins/2 .. bins/2 + PAD - 1 of each row) never hold a counter
    assert np.all((w % wps) < bins // 2)
    # the shared histogram fits its allocation: bins * (bins/2 + PAD) words
    assert w.max() < bins * wps


@pytest.mark.parametrize("bins", [2, 32, 128, 200, 224])
def test_wide_index_maps_back(bins):
    r, c = np.meshgrid(np.arange(bins), np.arange(bins), indexing="ij")
    logical = r * bins + c
    padded = r * (bins + 1) + c
    # the bin pass reads logical index idx at idx + row
    assert np.array_equal(padded, logical + logical // bins)
    assert padded.max() < bins * (bins + 1)


def test_padding_spreads_a_column_over_banks():
    """32 lanes whose voxels share the column bin (field 2) but differ in the
    row bin (field 1): unpadded, a 256-bin row is 128 words, a multiple of the
    32 banks, so all 32 words sit in one bank; with 3 pad words (131 per row)
    they sit in 32 different banks."""
    bins = 256
    lanes = np.arange(32)
    rows, cols = 100 + lanes, np.full(32, 61)
    plain = ((rows * bins + cols) >> 1) % 32
    padded = (packed_index(rows, cols, bins) >> 1) % 32
    assert len(set(plain.tolist())) == 1
    assert len(set(padded.tolist())) == 32
