"""Python binding of the GB300 isosurface-similarity engine (libisosim.so).

A thin ctypes layer over the C ABI declared in include/isosim.h.  Arrays are
numpy (host memory) or any object exposing ``data_ptr()`` (a device tensor);
the library reads either through cudaMemcpyDefault.  There is no fallback: if
the shared library is missing, importing this module raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libisosim.so")

ISO_OK = 0
ISO_ERR_ARG = -1
ISO_ERR_CUDA = -2
ISO_ERR_CAPACITY = -3
ISO_ERR_NOMEM = -4
ISO_ERR_INTERNAL = -5

SURFACE_MC = 0
SURFACE_APPROX = 1
FRAME_REF = 0
FRAME_CANON = 1
DF_BRUTE = 0
DF_LBVH = 1
DF_TC = 2
MI_FP64 = 0
MI_REF32 = 1
SERVE_FIFO = 0
SERVE_SHORTEST_FIRST = 1
MC_REF_DROPPED = 1


class IsoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("isosim error %d: %s" % (code, msg))
        self.code = code


class Opts(C.Structure):
    _fields_ = [("surface", C.c_int), ("frame", C.c_int), ("df_method", C.c_int),
                ("df_downscale", C.c_int), ("bins", C.c_int)]


class SurfaceStats(C.Structure):
    _fields_ = [("points", C.c_int64), ("active_voxels", C.c_int64), ("total_verts", C.c_int64),
                ("flags", C.c_int32), ("reserved", C.c_int32)]


class Rep(C.Structure):
    _fields_ = [("isovalue", C.c_float), ("priority", C.c_float), ("id", C.c_int32), ("map_id", C.c_int32)]


class Timing(C.Structure):
    _fields_ = [("surface_ms", C.c_float), ("distance_ms", C.c_float), ("histogram_ms", C.c_float),
                ("total_ms", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("hist_segment_values", C.c_int64), ("lbvh_group_points", C.c_int64), ("query_run", C.c_int32),
                ("from_cache", C.c_int32), ("default_ms", C.c_float), ("tuned_ms", C.c_float),
                ("trials", C.c_int32), ("reserved", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("X", C.c_int), ("Y", C.c_int), ("Z", C.c_int),
                ("isovalues", C.c_void_p), ("n", C.c_int), ("opts", Opts), ("ism_out", C.c_void_p),
                ("field_ids_out", C.c_void_p), ("m_out", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("m", C.c_int32), ("latency_ms", C.c_double), ("queue_ms", C.c_double),
                ("timing", Timing)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("failed", C.c_int64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("peak_device_bytes", C.c_size_t), ("held_device_bytes", C.c_size_t)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libisosim.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sig = {
        "iso_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
        "iso_ctx_destroy": (None, [P]),
        "iso_ctx_stream": (P, [P]),
        "iso_ctx_device_bytes": (C.c_size_t, [P]),
        "iso_ctx_launches": (C.c_int64, [P]),
        "iso_ctx_set_limit": (C.c_int, [P, C.c_int, C.c_int64]),
        "iso_last_error": (C.c_char_p, []),
        "iso_ism": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, P, C.c_int, C.POINTER(Opts), P, P,
                              C.POINTER(C.c_int32), P, C.POINTER(Timing)]),
        "iso_cross_map": (C.c_int, [P, P, P, C.c_int, C.c_int64, C.c_int, P]),
        "iso_surface_points": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_int, P, P,
                                         C.c_int64, P]),
        "iso_distance_field": (C.c_int, [P, P, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P]),
        "iso_similarity_map": (C.c_int, [P, P, C.c_int, C.c_int64, C.c_int, P, P]),
        "iso_select_representatives": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
        "iso_isovalues": (C.c_int, [P, P, C.c_int64, C.c_float, C.c_float, C.c_int, C.c_int, P]),
        "iso_real_range": (C.c_int, [P, P, C.c_int64, C.c_float, C.c_float, C.POINTER(C.c_float),
                                     C.POINTER(C.c_float)]),
        "calculate_histogram_h": (None, [P, P, P, C.c_int, C.c_ulong, C.c_ulong, P, P, P, P, C.c_int, C.c_bool]),
        "approximate_isosurfaces_h": (C.c_long, [P, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, P]),
        "iso_marching_cube_h": (C.c_int, [C.c_float, C.c_int, C.c_int, C.c_int, P, C.c_int, P, C.POINTER(C.c_long)]),
        "iso_generate_hierarchy_h": (C.c_int, [P, C.c_long, C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int]),
        "iso_transpose_xfastest": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, P]),
        "iso_copy_field": (C.c_int, [P, C.c_int, P]),
        "iso_copy_joint_histogram": (C.c_int, [P, C.c_int, C.c_int, P]),
        "iso_autotune": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, P, C.c_int, C.POINTER(Opts), C.c_char_p,
                                   C.POINTER(Tuning)]),
        "iso_server_create": (C.c_int, [C.c_int, C.c_int, C.c_size_t, C.POINTER(P)]),
        "iso_server_submit": (C.c_int, [P, C.POINTER(Request), C.POINTER(C.c_int64)]),
        "iso_server_wait": (C.c_int, [P, C.c_int64, C.POINTER(RequestResult)]),
        "iso_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
        "iso_server_destroy": (None, [P]),
        "iso_server_set_policy": (C.c_int, [P, C.c_int, C.c_double]),
        "iso_server_set_limit": (C.c_int, [P, C.c_int, C.c_int64]),
        "iso_similarity_map_noalloc": (C.c_int, [P, C.c_int, C.c_int64, C.c_int64, C.c_int, P, P]),
        "iso_pair_map": (C.c_int, [P, P, C.c_int, C.c_int64, C.c_int64, C.c_int, P, C.c_int64, P]),
        "iso_probe_counter_rate": (C.c_int, [P, C.c_int, C.POINTER(C.c_double)]),
        "iso_probe_wait_timeout": (C.c_int, [P, C.c_int, C.c_int64, C.POINTER(C.c_int)]),
        "iso_block_similarity": (C.c_int, [P, P, C.c_int64, C.c_int, P, C.c_int64, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()
_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]


def last_error():
    return lib.iso_last_error().decode(errors="replace")


def _check(code):
    if code < 0:
        raise IsoError(code, last_error())
    return code


def _ptr(a):
    """Address of a numpy array or a tensor-like object (data_ptr())."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


def _f32(a):
    if hasattr(a, "data_ptr"):
        return a
    return np.ascontiguousarray(a, dtype=np.float32)


class Context:
    """An engine context on one GPU (its own stream and device arena)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        _check(lib.iso_ctx_create(device, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib.iso_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self):
        return lib.iso_ctx_stream(self.handle)

    @property
    def device_bytes(self):
        """Bytes the context's device arena holds."""
        return lib.iso_ctx_device_bytes(self.handle)

    def set_lbvh_group_points(self, points):
        _check(lib.iso_ctx_set_limit(self.handle, 1, int(points)))

    def set_hist_segment_values(self, values):
        """Fields longer than `values` use the segment-major histogram schedule (0: never)."""
        _check(lib.iso_ctx_set_limit(self.handle, 2, int(values)))

    def set_device_bytes_cap(self, nbytes):
        """Largest arena the context may hold (0: no cap); beyond it calls fail
        with ISO_ERR_NOMEM."""
        _check(lib.iso_ctx_set_limit(self.handle, 5, int(nbytes)))

    def set_mi_mode(self, mode):
        """MI_FP64 (default: accurate, symmetric) or MI_REF32 (the reference's
        own FP32 evaluation per ordered pair, bit for bit)."""
        _check(lib.iso_ctx_set_limit(self.handle, 4, int(mode)))

    def set_surf_block_count_bytes(self, nbytes):
        """Largest per-block vertex-count table marching cubes keeps between its
        passes (0: the write pass counts again)."""
        _check(lib.iso_ctx_set_limit(self.handle, 3, int(nbytes)))

    @property
    def launches(self):
        return int(lib.iso_ctx_launches(self.handle))

    @property
    def device_bytes(self):
        return int(lib.iso_ctx_device_bytes(self.handle))

    # ---- pipeline ---------------------------------------------------------
    def ism(self, volume, dims, isovalues, surface=SURFACE_MC, frame=FRAME_REF, df_method=DF_LBVH,
            downscale=1, bins=128, out=None):
        """volume: X*Y*Z floats in img order (numpy or device tensor).
        Returns (ism m x m, field ids, per-isovalue stats, timing)."""
        X, Y, Z = dims
        iso = np.ascontiguousarray(isovalues, dtype=np.float32)
        n = iso.size
        vol = _f32(volume)
        opts = Opts(surface, frame, df_method, downscale, bins)
        ism = out if out is not None else np.zeros(n * n, dtype=np.float32)
        ids = np.zeros(n, dtype=np.int32)
        m = C.c_int32()
        stats = (SurfaceStats * n)()
        timing = Timing()
        _check(lib.iso_ism(self.handle, _ptr(vol), X, Y, Z, _ptr(iso), n, C.byref(opts), _ptr(ism), _ptr(ids),
                           C.byref(m), C.cast(stats, C.c_void_p), C.byref(timing)))
        mm = m.value
        if out is None:
            ism = ism[: mm * mm].reshape(mm, mm)
        return ism, ids[:mm], stats, timing

    def cross_map(self, fields_a, fields_b, bins=128):
        a = _f32(fields_a)
        b = _f32(fields_b)
        m, n = a.shape
        out = np.zeros((m, m), dtype=np.float32)
        _check(lib.iso_cross_map(self.handle, _ptr(a), _ptr(b), m, n, bins, _ptr(out)))
        return out

    def pair_map(self, fields, pairs, bins=128, n=None, stride=None, out=None):
        """NMI of every (a, b) in `pairs` over the rows of `fields` (R x stride).
        Returns the R x R map (entries outside the pairs stay as `out` had them)."""
        f = _f32(fields)
        R = f.shape[0]
        stride = stride or f.shape[1]
        n = n or stride
        p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        if out is None:
            out = np.zeros((R, R), dtype=np.float32)
        _check(lib.iso_pair_map(self.handle, _ptr(f), R, n, stride, bins, _ptr(p), p.shape[0], _ptr(out)))
        return out

    def block_similarity(self, pmap, k, blocks):
        """(mean, best-match) per k x k block (A, B) of a pair map."""
        m = _f32(pmap)
        R = m.shape[0]
        b = np.ascontiguousarray(blocks, dtype=np.int32).reshape(-1, 2)
        out = np.zeros((b.shape[0], 2), dtype=np.float32)
        _check(lib.iso_block_similarity(self.handle, _ptr(m), R, k, _ptr(b), b.shape[0], _ptr(out)))
        return out

    def counter_rate(self, bins=256):
        """Peak histogram counter updates per second (calibration kernel)."""
        r = C.c_double()
        _check(lib.iso_probe_counter_rate(self.handle, bins, C.byref(r)))
        return r.value

    def probe_wait_timeout(self, arrive, limit_ns):
        """Runs the kernels' bounded barrier wait on a barrier that one thread
        arrives at first (arrive) or that nothing arrives at; True when the
        wait gave up after limit_ns."""
        r = C.c_int()
        _check(lib.iso_probe_wait_timeout(self.handle, 1 if arrive else 0, int(limit_ns), C.byref(r)))
        return r.value == 1

    def copy_field(self, row, out):
        """Row `row` of the last ism() call's distance-field matrix into `out`."""
        _check(lib.iso_copy_field(self.handle, row, _ptr(out)))
        return out

    def autotune(self, volume, dims, isovalues, surface=SURFACE_MC, frame=FRAME_REF, df_method=DF_LBVH,
                 downscale=1, bins=128, cache_path=None):
        """Chooses and applies the fastest launch shapes for this workload
        (see iso_autotune); returns the Tuning record."""
        X, Y, Z = dims
        iso = np.ascontiguousarray(isovalues, dtype=np.float32)
        vol = _f32(volume)
        opts = Opts(surface, frame, df_method, downscale, bins)
        t = Tuning()
        _check(lib.iso_autotune(self.handle, _ptr(vol), X, Y, Z, _ptr(iso), iso.size, C.byref(opts),
                                cache_path.encode() if cache_path else None, C.byref(t)))
        return t

    def set_hist_row_codes(self, on):
        """Segment-major histograms with precomputed row buckets (1) or not (0)."""
        _check(lib.iso_ctx_set_limit(self.handle, 7, int(on)))

    def set_query_run(self, run):
        """LBVH query samples per lane along x (0: by volume size)."""
        _check(lib.iso_ctx_set_limit(self.handle, 6, int(run)))

    def joint_histogram(self, i, j, bins):
        """Joint histogram of ordered pair (i, j) kept by the last MI_REF32 map."""
        out = np.zeros((bins, bins), dtype=np.uint32)
        _check(lib.iso_copy_joint_histogram(self.handle, i, j, _ptr(out)))
        return out

    # ---- stages -----------------------------------------------------------
    def surface_points(self, volume, dims, isovalues, surface=SURFACE_MC, frame=FRAME_REF):
        """Returns (list of (P_k, 3) float32 arrays, stats)."""
        X, Y, Z = dims
        iso = np.ascontiguousarray(np.atleast_1d(isovalues), dtype=np.float32)
        n = iso.size
        vol = _f32(volume)
        counts = np.zeros(n, dtype=np.int64)
        stats = (SurfaceStats * n)()
        _check(lib.iso_surface_points(self.handle, _ptr(vol), X, Y, Z, _ptr(iso), n, surface, frame, _ptr(counts),
                                      None, 0, C.cast(stats, C.c_void_p)))
        total = int(counts.sum())
        pts = np.zeros((max(total, 1), 3), dtype=np.float32)
        _check(lib.iso_surface_points(self.handle, _ptr(vol), X, Y, Z, _ptr(iso), n, surface, frame, _ptr(counts),
                                      _ptr(pts), total, None))
        out, o = [], 0
        for c in counts:
            out.append(pts[o:o + c].copy())
            o += c
        return out, stats

    def distance_field(self, points, dims, downscale=1, method=DF_LBVH):
        X, Y, Z = dims
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        F = (X // downscale) * (Y // downscale) * (Z // downscale)
        out = np.zeros(F, dtype=np.float32)
        _check(lib.iso_distance_field(self.handle, _ptr(p), p.shape[0], X, Y, Z, downscale, method, _ptr(out)))
        return out

    def similarity_map(self, fields, bins=128, joint=False):
        f = _f32(fields)
        m, n = f.shape
        ism = np.zeros((m, m), dtype=np.float32)
        jh = np.zeros((m, m, bins, bins), dtype=np.uint32) if joint else None
        _check(lib.iso_similarity_map(self.handle, _ptr(f), m, n, bins, _ptr(ism), _ptr(jh)))
        return (ism, jh) if joint else ism

    def real_range(self, volume, cfg_min=-1e30, cfg_max=1e30):
        vol = _f32(volume)
        lo, hi = C.c_float(), C.c_float()
        n = vol.numel() if hasattr(vol, "numel") else vol.size
        _check(lib.iso_real_range(self.handle, _ptr(vol), n, cfg_min, cfg_max, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def isovalues(self, volume, vmin, vmax, n, uniform=True):
        vol = _f32(volume) if volume is not None else None
        out = np.zeros(n, dtype=np.float32)
        size = 0 if vol is None else (vol.numel() if hasattr(vol, "numel") else vol.size)
        _check(lib.iso_isovalues(self.handle, _ptr(vol), size, vmin, vmax, n, 1 if uniform else 0, _ptr(out)))
        return out


class Server:
    """Device-resident request loop: `slots` concurrent workers under an HBM budget."""

    def __init__(self, device=0, slots=4, budget_bytes=150 << 30):
        h = C.c_void_p()
        _check(lib.iso_server_create(device, slots, budget_bytes, C.byref(h)))
        self.handle = h
        self._live = {}

    def submit(self, volume, dims, isovalues, surface=SURFACE_MC, frame=FRAME_REF, df_method=DF_LBVH,
               downscale=1, bins=128):
        X, Y, Z = dims
        vol = _f32(volume)
        iso = np.ascontiguousarray(isovalues, dtype=np.float32)
        n = iso.size
        ism = np.zeros(n * n, dtype=np.float32)
        ids = np.zeros(n, dtype=np.int32)
        m = np.zeros(1, dtype=np.int32)
        req = Request(_ptr(vol), X, Y, Z, _ptr(iso), n, Opts(surface, frame, df_method, downscale, bins),
                      _ptr(ism), _ptr(ids), _ptr(m))
        t = C.c_int64()
        _check(lib.iso_server_submit(self.handle, C.byref(req), C.byref(t)))
        self._live[t.value] = (vol, iso, ism, ids, m)
        return t.value

    def wait(self, ticket):
        """Returns (ism m x m, ids, RequestResult)."""
        res = RequestResult()
        rc = lib.iso_server_wait(self.handle, ticket, C.byref(res))
        vol, iso, ism, ids, m = self._live.pop(ticket)
        _check(rc)
        mm = res.m
        return ism[: mm * mm].reshape(mm, mm), ids[:mm], res

    def set_policy(self, policy, max_wait_ms=0.0):
        """SERVE_FIFO or SERVE_SHORTEST_FIRST (smallest work estimate first,
        the oldest request first once it waited max_wait_ms)."""
        _check(lib.iso_server_set_policy(self.handle, int(policy), float(max_wait_ms)))

    def set_limit(self, which, value):
        """iso_ctx_set_limit on every worker context (only while idle)."""
        _check(lib.iso_server_set_limit(self.handle, int(which), int(value)))

    def set_mi_mode(self, mode):
        """MI_FP64 or MI_REF32 for every request (only while idle)."""
        self.set_limit(4, mode)

    def stats(self):
        st = ServerStats()
        _check(lib.iso_server_get_stats(self.handle, C.byref(st)))
        return st

    def close(self):
        if self.handle:
            lib.iso_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def select_representatives(ism, ids, isovalues, cnt=16):
    ism = np.ascontiguousarray(ism, dtype=np.float32)
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    iso = np.ascontiguousarray(isovalues, dtype=np.float32)
    m = ism.shape[0]
    out = (Rep * max(cnt, 1))()
    k = _check(lib.iso_select_representatives(_ptr(ism), m, _ptr(ids), _ptr(iso), cnt, C.cast(out, C.c_void_p)))
    return [(out[i].isovalue, out[i].priority, out[i].id, out[i].map_id) for i in range(k)]


# ---- reference-named drop-in functions (the current CUDA device) -------------

def calculate_histogram_h(fields, mins, maxs, bins, sim_size=None, multi=False):
    """Calls the reference-named entry (the reference's FP32 map, bit for bit).
    fields: list of 1-D float32 arrays."""
    fields = [np.ascontiguousarray(f, dtype=np.float32) for f in fields]
    nf = len(fields) // 2 if multi else len(fields)
    n = fields[0].size
    sim_size = sim_size or nf
    arr = (C.c_void_p * len(fields))(*[f.ctypes.data for f in fields])
    mins = np.ascontiguousarray(mins, dtype=np.float32)
    maxs = np.ascontiguousarray(maxs, dtype=np.float32)
    sim = np.zeros((sim_size, sim_size), dtype=np.float32)
    cols = np.zeros(nf * nf * bins, dtype=np.uint32)
    rows = np.zeros(nf * nf * bins, dtype=np.uint32)
    lib.calculate_histogram_h(C.cast(arr, C.c_void_p), _ptr(mins), _ptr(maxs), n, nf, bins, None, _ptr(cols),
                              _ptr(rows), _ptr(sim), sim_size, multi)
    err = last_error()
    if err:
        raise IsoError(ISO_ERR_CUDA, err)
    return sim, cols.reshape(nf, nf, bins), rows.reshape(nf, nf, bins)


def approximate_isosurfaces_h(volume, dims, iso):
    X, Y, Z = dims
    vol = np.ascontiguousarray(volume, dtype=np.float32)
    out = C.c_void_p()
    n = _check(lib.approximate_isosurfaces_h(_ptr(vol), iso, X, Y, Z, 1, C.byref(out)))
    arr = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_int32)), shape=(max(n, 1) * 3,))[: n * 3].copy()
    _libc.free(out)
    return arr.reshape(n, 3)


def marching_cube_h(volume, dims, iso, max_verts=None):
    X, Y, Z = dims
    vol = np.ascontiguousarray(volume, dtype=np.float32)
    out = C.c_void_p()
    cnt = C.c_long()
    _check(lib.iso_marching_cube_h(iso, X, Y, Z, _ptr(vol), max_verts or X * Y * Z, C.byref(out), C.byref(cnt)))
    n = cnt.value
    arr = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_float)), shape=(max(n, 1) * 4,))[: n * 4].copy()
    _libc.free(out)
    return arr.reshape(n, 4)


def generate_hierarchy_h(points, dims, downscale=1, num_samples=1500):
    X, Y, Z = dims
    p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((X // downscale) * (Y // downscale) * (Z // downscale), dtype=np.float32)
    _check(lib.iso_generate_hierarchy_h(_ptr(p), p.shape[0], X, Y, Z, _ptr(out), num_samples, downscale))
    return out
