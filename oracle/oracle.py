"""ctypes binding of the CPU oracle (liboracle.so) and of the reference harness
(_ref/libisoref.so, built from the reference's own sources where available).

TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and bench.py's CPU
baseline as the checker.  Nothing in the engine imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libisoref.so")

_P = C.c_void_p


def build():
    """Compiles liboracle.so with the Makefile beside this file."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Rep(C.Structure):
    _fields_ = [("isovalue", C.c_float), ("priority", C.c_float), ("id", C.c_int32), ("map_id", C.c_int32)]


def _load_oracle():
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "isooracle.c")):
        build()
    lib = C.CDLL(ORACLE_SO)
    sig = {
        "orc_find_bucket": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_int]),
        "orc_field_interval": (None, [_P, C.c_long, _P, _P]),
        "orc_pair_histogram": (None, [_P, _P, C.c_long, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, _P, _P, _P]),
        "orc_mi_f32": (C.c_float, [_P, C.c_int, C.c_float, _P, _P]),
        "orc_mi_f64": (C.c_double, [_P, C.c_int, C.c_double]),
        "orc_similarity_map": (None, [_P, C.c_int, C.c_long, C.c_int, C.c_int, _P]),
        "orc_approximation": (C.c_long, [_P, C.c_int, C.c_int, C.c_int, C.c_float, _P, C.c_long]),
        "orc_mc_vertex_counts": (None, [_P]),
        "orc_mc_classified_voxels": (C.c_long, [C.c_long]),
        "orc_marching_cubes": (C.c_long, [_P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, _P, C.c_long, _P]),
        "orc_normalize_points": (None, [_P, C.c_long, C.c_int, C.c_int, C.c_int, _P]),
        "orc_distance_field_f32": (None, [_P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
        "orc_distance_field_f64": (None, [_P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
        "orc_distance_field_kd": (None, [_P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, _P, C.c_long, _P]),
        "orc_distance_field_kd_timed": (None, [_P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, _P, C.c_long, _P,
                                               _P, _P]),
        "orc_real_range": (None, [_P, C.c_long, C.c_float, C.c_float, _P, _P]),
        "orc_isovalues": (None, [_P, C.c_long, C.c_float, C.c_float, C.c_int, C.c_int, _P]),
        "orc_select_representatives": (C.c_int, [_P, C.c_int, _P, _P, C.c_int, _P]),
        "orc_ref_morton": (None, [_P, C.c_long, _P]),
        "orc_ref_lbvh": (C.c_long, [_P, C.c_long, _P, _P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


orc = _load_oracle()


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def find_bucket(v, mn, step, bins):
    return orc.orc_find_bucket(v, mn, step, bins)


def field_interval(f):
    f = f32(f)
    lo, hi = np.zeros(1, np.float32), np.zeros(1, np.float32)
    orc.orc_field_interval(_p(f), f.size, _p(lo), _p(hi))
    return float(lo[0]), float(hi[0])


def pair_histogram(f1, f2, bins, interval1=None, interval2=None):
    f1, f2 = f32(f1), f32(f2)
    i1 = interval1 or field_interval(f1)
    i2 = interval2 or field_interval(f2)
    joint = np.zeros((bins, bins), np.uint32)
    cs = np.zeros(bins, np.uint32)
    rs = np.zeros(bins, np.uint32)
    orc.orc_pair_histogram(_p(f1), _p(f2), f1.size, i1[0], i1[1], i2[0], i2[1], bins, _p(joint), _p(cs), _p(rs))
    return joint, cs, rs


def mi_f32(joint, col_sums, row_sums, n):
    j = np.ascontiguousarray(joint, np.uint32)
    return orc.orc_mi_f32(_p(j), j.shape[0], float(n), _p(np.ascontiguousarray(col_sums, np.uint32)),
                          _p(np.ascontiguousarray(row_sums, np.uint32)))


def mi_f64(joint, n):
    j = np.ascontiguousarray(joint, np.uint32)
    return orc.orc_mi_f64(_p(j), j.shape[0], float(n))


def similarity_map(fields, bins, mode=0):
    """mode 0: FP64 MI on unordered pairs (mirrored); mode 1: FP32 reference MI on ordered pairs."""
    f = f32(fields)
    m, n = f.shape
    out = np.zeros((m, m), np.float32)
    orc.orc_similarity_map(_p(f), m, n, bins, mode, _p(out))
    return out


def approximation(vol, dims, iso):
    X, Y, Z = dims
    v = f32(vol)
    cap = (X - 1) * (Y - 1) * (Z - 1)
    out = np.zeros((max(cap, 1), 3), np.int32)
    n = orc.orc_approximation(_p(v), X, Y, Z, iso, _p(out), cap)
    return out[:n].copy()


def mc_vertex_counts():
    out = np.zeros(256, np.uint32)
    orc.orc_mc_vertex_counts(_p(out))
    return out


def marching_cubes(vol, dims, iso, frame=0, cap=None):
    X, Y, Z = dims
    v = f32(vol)
    stats = np.zeros(2, np.int64)
    n = orc.orc_marching_cubes(_p(v), X, Y, Z, iso, frame, None, 0, _p(stats))
    out = np.zeros((max(n, 1), 3), np.float32)
    orc.orc_marching_cubes(_p(v), X, Y, Z, iso, frame, _p(out), n, _p(stats))
    return out[:n].copy(), int(stats[0]), int(stats[1])


def normalize_points(pts, dims):
    p = f32(pts).reshape(-1, 3)
    out = np.zeros_like(p)
    orc.orc_normalize_points(_p(p), p.shape[0], dims[0], dims[1], dims[2], _p(out))
    return out


def distance_field_f32(pts_norm, dims, ds=1):
    p = f32(pts_norm).reshape(-1, 3)
    X, Y, Z = dims
    out = np.zeros((X // ds) * (Y // ds) * (Z // ds), np.float32)
    orc.orc_distance_field_f32(_p(p), p.shape[0], X, Y, Z, ds, _p(out))
    return out


def distance_field_kd(pts_norm, dims, ds=1, idx=None):
    """Canonical FP32 field through a k-d tree (bit-identical to distance_field_f32)."""
    p = f32(pts_norm).reshape(-1, 3)
    X, Y, Z = dims
    if idx is None:
        out = np.zeros((X // ds) * (Y // ds) * (Z // ds), np.float32)
        orc.orc_distance_field_kd(_p(p), p.shape[0], X, Y, Z, ds, None, 0, _p(out))
    else:
        idx = np.ascontiguousarray(idx, np.int64)
        out = np.zeros(idx.size, np.float32)
        orc.orc_distance_field_kd(_p(p), p.shape[0], X, Y, Z, ds, _p(idx), idx.size, _p(out))
    return out


def distance_field_kd_timed(pts_norm, dims, idx, ds=1):
    """distance_field_kd on sample indices idx; returns (field values, tree
    build seconds, query seconds), timed inside the C code."""
    p = f32(pts_norm).reshape(-1, 3)
    X, Y, Z = dims
    idx = np.ascontiguousarray(idx, np.int64)
    out = np.zeros(idx.size, np.float32)
    tb, tq = np.zeros(1), np.zeros(1)
    orc.orc_distance_field_kd_timed(_p(p), p.shape[0], X, Y, Z, ds, _p(idx), idx.size, _p(out), _p(tb), _p(tq))
    return out, float(tb[0]), float(tq[0])


def distance_field_f64(pts_norm, dims, ds=1):
    p = f32(pts_norm).reshape(-1, 3)
    X, Y, Z = dims
    out = np.zeros((X // ds) * (Y // ds) * (Z // ds), np.float64)
    orc.orc_distance_field_f64(_p(p), p.shape[0], X, Y, Z, ds, _p(out))
    return out


def real_range(vol, cfg_min, cfg_max):
    v = f32(vol)
    lo, hi = np.zeros(1, np.float32), np.zeros(1, np.float32)
    orc.orc_real_range(_p(v), v.size, cfg_min, cfg_max, _p(lo), _p(hi))
    return float(lo[0]), float(hi[0])


def isovalues(vol, vmin, vmax, n, uniform=True):
    v = f32(vol)
    out = np.zeros(n, np.float32)
    orc.orc_isovalues(_p(v), v.size, vmin, vmax, n, 1 if uniform else 0, _p(out))
    return out


def select_representatives(ism, ids, isos, cnt=16):
    ism = f32(ism)
    ids = np.ascontiguousarray(ids, np.int32)
    isos = f32(isos)
    out = (Rep * max(cnt, 1))()
    k = orc.orc_select_representatives(_p(ism), ism.shape[0], _p(ids), _p(isos), cnt, C.cast(out, C.c_void_p))
    return [(out[i].isovalue, out[i].priority, out[i].id, out[i].map_id) for i in range(k)]


# ---- the reference's own functions (only where oracle/_ref was built) -------

def reference_root():
    """Where oracle/build_ref.sh found the reference's sources, or None (the
    file exists only where they were present when the checkers were built)."""
    path = os.path.join(os.path.dirname(REF_SO), "reference_root.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        root = f.read().strip()
    return root if os.path.isdir(root) else None


def load_reference():
    """Returns the reference harness library, or None if it was not built."""
    if not os.path.exists(REF_SO):
        return None
    try:
        lib = C.CDLL(REF_SO)
    except OSError:
        return None
    lib.ref_mutual_information.restype = C.c_float
    lib.ref_mutual_information.argtypes = [_P, C.c_int, C.c_float, _P, _P]
    lib.ref_find_bucket.restype = C.c_int
    lib.ref_find_bucket.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int]
    lib.ref_similarity_map_cpu.restype = C.c_int
    lib.ref_similarity_map_cpu.argtypes = [_P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P]
    lib.ref_approximation_cpu.restype = C.c_long
    lib.ref_approximation_cpu.argtypes = [_P, C.c_float, C.c_int, C.c_int, C.c_int, _P, C.c_long]
    return lib


def ref_similarity_map(ref, fields, bins, multi=False, threads=1, want_sums=False):
    """The reference's calculate_histogram_CPU over every ordered pair (FP32 MI)."""
    fl = [f32(f) for f in fields]
    nf = len(fl) // 2 if multi else len(fl)
    n = fl[0].size
    arr = (C.c_void_p * len(fl))(*[f.ctypes.data for f in fl])
    sim = np.zeros((nf, nf), np.float32)
    cols = np.zeros(nf * nf * bins, np.uint32) if want_sums else None
    rows = np.zeros(nf * nf * bins, np.uint32) if want_sums else None
    ref.ref_similarity_map_cpu(C.cast(arr, C.c_void_p), n, nf, bins, 1 if multi else 0, threads, _p(sim), None,
                               _p(cols), _p(rows))
    if want_sums:
        return sim, cols.reshape(nf, nf, bins), rows.reshape(nf, nf, bins)
    return sim


def ref_approximation(ref, vol, dims, iso):
    X, Y, Z = dims
    v = f32(vol)
    cap = (X - 1) * (Y - 1) * (Z - 1)
    out = np.zeros((max(cap, 1), 3), np.int32)
    n = ref.ref_approximation_cpu(_p(v), iso, X, Y, Z, _p(out), cap)
    return out[:n].copy()


def ref_morton(pts):
    """The reference's 30-bit Morton codes of float32 points (BVH.cu:86-106)."""
    p = f32(pts).reshape(-1, 3)
    out = np.zeros(p.shape[0], np.uint32)
    orc.orc_ref_morton(_p(p), p.shape[0], _p(out))
    return out


def ref_lbvh(sorted_codes):
    """The reference's tree over sorted Morton codes (BVH.cu:122-345):
    (left, right, depth) with leaves encoded -(index) - 1; depth -1 when the
    rules do not give a tree."""
    c = np.ascontiguousarray(sorted_codes, np.uint32)
    n = c.size
    left = np.zeros(max(n - 1, 1), np.int32)
    right = np.zeros(max(n - 1, 1), np.int32)
    depth = orc.orc_ref_lbvh(_p(c), n, _p(left), _p(right))
    return left[:n - 1], right[:n - 1], int(depth)
