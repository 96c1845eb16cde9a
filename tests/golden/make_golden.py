"""Regenerates the golden vectors in this folder from the reference's own code.

Needs oracle/_ref/libisoref.so, which oracle/build_ref.sh compiles from the
reference sources (only possible where the reference tree is present).  The
vectors pin the CPU oracle on machines where the reference is absent.

    python tests/golden/make_golden.py

Produces:
  bucket_mi.npz      findBucket_d on seeded and edge-case inputs; the
                     reference's FP32 calculateMutualInformation of seeded
                     joint histograms
  simmap_small.npz   calculate_histogram_CPU over every ordered pair of five
                     seeded fields (similarity map, column and row sums)
  approx_small.npz   calculate_approximation_CPU cells of a seeded 13x11x9
                     volume at three isovalues
  mc_table.npz       SHA-256 of the reference's per-case triangle-vertex table
                     (the table itself is not copied)
"""
import hashlib
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402

_REF_ROOT = oracle.reference_root()
REF_TABLES = os.path.join(_REF_ROOT, "isosurfaces_lib", "isosurfaces_cuda", "src", "tables.h") if _REF_ROOT else None


def bucket_mi(ref):
    rng = np.random.default_rng(11)
    vals = rng.uniform(0, 2, 400).astype(np.float32)
    mins = rng.uniform(0, 0.5, 400).astype(np.float32)
    steps = rng.uniform(1e-3, 0.05, 400).astype(np.float32)
    bins = rng.choice([16, 128, 256], 400).astype(np.int32)
    # edge cases: zero step, value at max, exact multiples of the step
    vals[:4] = [0.5, 1.0, 0.25, 3.0]
    mins[:4] = [0.5, 0.0, 0.0, 0.0]
    steps[:4] = [0.0, np.float32(1.0) / 128, np.float32(0.25) / 16, np.float32(1.0) / 256]
    buckets = np.array([ref.ref_find_bucket(float(v), float(m), float(s), int(b))
                        for v, m, s, b in zip(vals, mins, steps, bins)], np.int32)
    hists, mis = [], []
    for k in range(6):
        h = rng.integers(0, 50, size=(32, 32)).astype(np.uint32)
        h[rng.uniform(size=(32, 32)) < 0.6] = 0
        if k == 0:
            h = np.diag(rng.integers(1, 9, size=32)).astype(np.uint32)
        n = int(h.sum())
        cs = np.ascontiguousarray(h.sum(axis=0), np.uint32)
        rs = np.ascontiguousarray(h.sum(axis=1), np.uint32)
        hh = np.ascontiguousarray(h)
        mis.append(ref.ref_mutual_information(hh.ctypes.data, 32, float(n), cs.ctypes.data, rs.ctypes.data))
        hists.append(hh)
    np.savez_compressed(os.path.join(HERE, "bucket_mi.npz"), vals=vals, mins=mins, steps=steps, bins=bins,
                        buckets=buckets, hists=np.stack(hists), mis=np.array(mis, np.float32))


def simmap_small(ref):
    rng = np.random.default_rng(12)
    n = 5003
    base = rng.uniform(0, 1, n)
    fields = [np.abs(base * (1 + 0.3 * k) + 0.2 * rng.standard_normal(n)).astype(np.float32) for k in range(5)]
    sim, cols, rows = oracle.ref_similarity_map(ref, fields, 32, want_sums=True)
    np.savez_compressed(os.path.join(HERE, "simmap_small.npz"), fields=np.stack(fields), bins=32, sim=sim,
                        cols=cols, rows=rows)


def approx_small(ref):
    rng = np.random.default_rng(13)
    dims = (13, 11, 9)
    vol = rng.standard_normal(dims).astype(np.float32)
    isos = np.array([-0.5, 0.0, 0.7], np.float32)
    cells = [oracle.ref_approximation(ref, vol, dims, float(i)) for i in isos]
    np.savez_compressed(os.path.join(HERE, "approx_small.npz"), vol=vol, dims=np.array(dims), isos=isos,
                        counts=np.array([len(c) for c in cells]), cells=np.concatenate(cells))


def mc_table():
    src = open(REF_TABLES).read()
    body = src[src.index("numVertsTable[256]"):]
    body = body[body.index("{") + 1: body.index("}")]
    vals = np.array([int(x) for x in re.findall(r"\d+", body)], np.uint32)
    assert vals.size == 256
    digest = hashlib.sha256(vals.tobytes()).hexdigest()
    np.savez_compressed(os.path.join(HERE, "mc_table.npz"), sha256=np.array(digest))


def main():
    ref = oracle.load_reference()
    if ref is None:
        sys.exit("oracle/_ref/libisoref.so is missing: run oracle/build_ref.sh first")
    bucket_mi(ref)
    simmap_small(ref)
    approx_small(ref)
    mc_table()
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
