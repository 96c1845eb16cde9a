"""The CPU oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py) and, where it was built, against the reference
harness directly."""
import hashlib
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
_REF_ROOT = oracle.reference_root()
REF_TABLES = os.path.join(_REF_ROOT, "isosurfaces_lib", "isosurfaces_cuda", "src", "tables.h") if _REF_ROOT else None


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_bucket_matches_reference_golden():
    g = load("bucket_mi.npz")
    got = [oracle.find_bucket(float(v), float(m), float(s), int(b))
           for v, m, s, b in zip(g["vals"], g["mins"], g["steps"], g["bins"])]
    assert np.array_equal(np.array(got, np.int32), g["buckets"])


def test_mi_f32_matches_reference_golden_bitwise():
    g = load("bucket_mi.npz")
    for h, want in zip(g["hists"], g["mis"]):
        n = int(h.sum())
        got = oracle.mi_f32(h, h.sum(axis=0).astype(np.uint32), h.sum(axis=1).astype(np.uint32), n)
        assert np.float32(got) == want


def test_mi_f64_close_to_reference_fp32():
    g = load("bucket_mi.npz")
    for h, want in zip(g["hists"], g["mis"]):
        got = oracle.mi_f64(h, int(h.sum()))
        assert abs(got - float(want)) < 1e-5
    # identity histogram -> 1
    assert oracle.mi_f64(np.diag(np.arange(1, 9)).astype(np.uint32), 36) == pytest.approx(1.0, abs=1e-15)


def test_similarity_map_matches_reference_golden():
    g = load("simmap_small.npz")
    fields, bins = g["fields"], int(g["bins"])
    sim32 = oracle.similarity_map(fields, bins, mode=1)
    assert np.array_equal(sim32, g["sim"])  # FP32 restatement is bit-exact
    sim64 = oracle.similarity_map(fields, bins, mode=0)
    assert np.abs(sim64 - g["sim"]).max() < 2e-5
    m = fields.shape[0]
    for i in range(m):
        for j in range(m):
            lo_i, hi_i = oracle.field_interval(fields[i])
            lo_j, hi_j = oracle.field_interval(fields[j])
            joint, cs, rs = oracle.pair_histogram(fields[i], fields[j], bins, (lo_i, hi_i), (lo_j, hi_j))
            assert np.array_equal(cs, g["cols"][i, j])
            assert np.array_equal(rs, g["rows"][i, j])


def test_approximation_matches_reference_golden():
    g = load("approx_small.npz")
    dims = tuple(int(d) for d in g["dims"])
    off = 0
    for iso, cnt in zip(g["isos"], g["counts"]):
        got = oracle.approximation(g["vol"], dims, float(iso))
        assert np.array_equal(got, g["cells"][off:off + cnt])
        off += cnt


def test_mc_table_derivation_matches_reference_hash():
    g = load("mc_table.npz")
    derived = oracle.mc_vertex_counts().astype(np.uint32)
    assert hashlib.sha256(derived.tobytes()).hexdigest() == str(g["sha256"])


@pytest.mark.skipif(not REF_TABLES or not os.path.exists(REF_TABLES), reason="reference tree not present")
def test_mc_table_derivation_matches_reference_text():
    import re
    src = open(REF_TABLES).read()
    body = src[src.index("numVertsTable[256]"):]
    body = body[body.index("{") + 1: body.index("}")]
    want = np.array([int(x) for x in re.findall(r"\d+", body)], np.uint32)
    assert np.array_equal(oracle.mc_vertex_counts(), want)


def test_oracle_vs_reference_harness_random(ref):
    rng = np.random.default_rng(5)
    n = 20011
    fields = [np.abs(rng.standard_normal(n)).astype(np.float32) * (1 + k) for k in range(4)]
    want = oracle.ref_similarity_map(ref, fields, 64)
    got = oracle.similarity_map(np.stack(fields), 64, mode=1)
    assert np.array_equal(got, want)
    vol = rng.standard_normal((9, 8, 7)).astype(np.float32)
    for iso in (-1.0, 0.0, 0.3):
        assert np.array_equal(oracle.approximation(vol, (9, 8, 7), iso), oracle.ref_approximation(ref, vol, (9, 8, 7), iso))


def test_mc_oracle_kat_single_cells():
    """Every case code on a 2x2x2 volume: the unique vertices are the crossing
    edges' midpoints (values 0/1, iso 0.5) and the triangle-vertex total is the
    case's count (plus the clamped boundary cells' degenerate cases)."""
    counts = oracle.mc_vertex_counts()
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for case in range(256):
        vol = np.zeros((2, 2, 2), np.float32)  # canonical frame: vol[a, b, c]
        for k, (a, b, c) in enumerate(corner):
            vol[a, b, c] = 0.0 if (case >> k) & 1 else 1.0
        pts, active, total = oracle.marching_cubes(vol, (2, 2, 2), 0.5, frame=1)
        # cell (0,0,0) carries the case; cells at a/b/c == 1 see clamped corners
        assert total >= counts[case]
        if counts[case] == 0:
            assert len(pts) == 0
        else:
            assert np.all((pts * 2) == np.round(pts * 2))


def test_isovalues_linear_and_uniform():
    rng = np.random.default_rng(3)
    vol = rng.standard_normal(4096).astype(np.float32)
    lo, hi = oracle.real_range(vol, -1e9, 1e9)
    assert lo == vol.min() and hi == vol.max()
    lin = oracle.isovalues(vol, lo, hi, 8, uniform=False)
    step = np.float32((np.float32(hi) - np.float32(lo)) / np.float32(8))
    assert np.array_equal(lin, (np.float32(lo) + step * np.arange(8, dtype=np.float32)).astype(np.float32))
    eq = oracle.isovalues(vol, lo, hi, 8, uniform=True)
    assert np.all(np.diff(eq) > 0)
