"""The reference's own GPU kernels -- its joint histogram and its marching
cubes -- run on this machine's GPU (test infrastructure only: a checker,
never the engine).  The marching-cubes harness is marching_cubes() below.

oracle/build_ref.sh compiles isosurfaces_cuda/src/JointHistogram.cu from the
reference's sources, device code only and with nvcc's default flags (as the
reference's CMake build passes none), into oracle/_ref/ref_histogram.cubin.
This module loads that cubin through the CUDA driver API (ctypes on
libcuda.so.1) and drives its kernel calculate_histogram_g (JointHistogram.cu:
100-162) the way the reference's host function calculate_histogram_h
(JointHistogram.cu:266-420) does for a single histogram run:

  * one task per ordered pair, (i, j) for i, j < m in row-major order, or
    (i, j + m) in multi mode (:306-328);
  * fields staged in chunks of MAX_PER_RUN = 1,000,000 values at stride
    MAX_PER_RUN (:383-394), one kernel launch per chunk, the last chunk
    flagged so the kernel evaluates calculateMutualInformation (:156-160);
  * the run-info values of calculateRunInfo (:231-264) for the case where all
    m*m histograms fit one allocation of MALLOC_MAX_BYTES (2 GiB,
    isosurfaces_cuda/hdr/common.h:8).

The result is the reference's own output on the GPU: its FP32 similarity map
(every ordered pair), its joint histograms, and its column and row sums.
Sizes that need several histogram runs, or whose last chunk would be empty
(the reference's loop skips a chunk when the field length is a multiple of
MAX_PER_RUN), are refused here rather than run.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_histogram.cubin")

MAX_PER_RUN = 1000000             # JointHistogram.cu:21
MALLOC_MAX_BYTES = 1 << 31        # isosurfaces_cuda/hdr/common.h:8
KERNEL = b"_Z21calculate_histogram_gPfS_S_PjS0_S0_P4int2mmS_7runInfo8dataInfo"


class RunInfo(C.Structure):
    """struct runInfo (JointHistogram.cu:77-90); LP64 layout, 88 bytes."""
    _fields_ = [("tasksPerRun", C.c_ulong), ("lastRunMemBytes", C.c_ulong), ("histMemMax", C.c_ulong),
                ("offsetMax", C.c_ulong), ("memoryPerRun", C.c_ulong), ("odd", C.c_bool),
                ("maxSize", C.c_ulong), ("fieldMaxMemory", C.c_ulong), ("fieldsLastRun", C.c_bool),
                ("fieldsLastRunBytes", C.c_ulong), ("multi", C.c_bool)]


class DataInfo(C.Structure):
    """struct dataInfo (JointHistogram.cu:92-98)."""
    _fields_ = [("fieldSize", C.c_int), ("histogramSize", C.c_int), ("numFields", C.c_int),
                ("similarityMapSize", C.c_int)]


assert C.sizeof(RunInfo) == 88 and C.sizeof(DataInfo) == 16


def available():
    return os.path.exists(CUBIN)


class _Driver:
    def __init__(self):
        cu = C.CDLL("libcuda.so.1")
        self.cu = cu
        self._check(cu.cuInit(0), "cuInit")
        dev = C.c_int()
        self._check(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
        ctx = C.c_void_p()
        # the device's primary context: the one the CUDA runtime (and the
        # engine) use, so device pointers pass freely between them
        self._check(cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self._check(cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.modules = {}
        self.fn = self.function(CUBIN, KERNEL)
        cu.cuMemAlloc_v2.argtypes = [C.POINTER(C.c_uint64), C.c_size_t]
        cu.cuMemFree_v2.argtypes = [C.c_uint64]
        cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        cu.cuMemcpyDtoH_v2.argtypes = [C.c_void_p, C.c_uint64, C.c_size_t]
        cu.cuMemsetD8_v2.argtypes = [C.c_uint64, C.c_ubyte, C.c_size_t]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("CUDA driver call %s failed with %d" % (what, rc))

    def alloc(self, nbytes):
        p = C.c_uint64()
        self._check(self.cu.cuMemAlloc_v2(C.byref(p), max(int(nbytes), 256)), "cuMemAlloc")
        return p.value

    def free(self, p):
        self.cu.cuMemFree_v2(p)

    def h2d(self, dst, arr):
        arr = np.ascontiguousarray(arr)
        self._check(self.cu.cuMemcpyHtoD_v2(dst, arr.ctypes.data, arr.nbytes), "cuMemcpyHtoD")

    def d2h(self, arr, src):
        self._check(self.cu.cuMemcpyDtoH_v2(arr.ctypes.data, src, arr.nbytes), "cuMemcpyDtoH")

    def memset0(self, p, nbytes):
        self._check(self.cu.cuMemsetD8_v2(p, 0, nbytes), "cuMemsetD8")

    def function(self, cubin, name):
        """A kernel of a cubin under oracle/_ref/ (each cubin loaded once)."""
        mod = self.modules.get(cubin)
        if mod is None:
            mod = C.c_void_p()
            self._check(self.cu.cuModuleLoad(C.byref(mod), cubin.encode()), "cuModuleLoad")
            self.modules[cubin] = mod
        fn = C.c_void_p()
        self._check(self.cu.cuModuleGetFunction(C.byref(fn), mod, name), "cuModuleGetFunction")
        return fn

    def launch(self, grid, block, args, fn=None):
        """grid: an int (x) or an (x, y) pair; one synchronising launch."""
        gx, gy = (grid, 1) if isinstance(grid, int) else grid
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(fn if fn is not None else self.fn, gx, gy, 1, block, 1, 1, 0, None,
                                           ptrs, None), "cuLaunchKernel")
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


_DRIVER = None


def _driver():
    global _DRIVER
    if _DRIVER is None:
        _DRIVER = _Driver()
    return _DRIVER


def similarity(fields, bins, mins=None, maxs=None, multi=False, block=128):
    """The reference's calculate_histogram_h on the GPU for m fields (2m rows
    in multi mode: the first m against the last m).  fields: [rows, F]
    float32.  mins/maxs: per-row interval (default: each row's min and max,
    the values DistanceField::getInterval gives for non-negative fields).
    Returns (sim [m, m] float32, joint [m*m, bins, bins] uint32,
    col_sums [m*m, bins], row_sums [m*m, bins])."""
    drv = _driver()
    fields = np.ascontiguousarray(fields, dtype=np.float32)
    rows, F = fields.shape
    m = rows // 2 if multi else rows
    if mins is None:
        mins = fields.min(axis=1)
        maxs = fields.max(axis=1)
    mins = np.ascontiguousarray(mins, np.float32)
    maxs = np.ascontiguousarray(maxs, np.float32)
    hist_bytes = m * m * bins * bins * 4
    if hist_bytes > MALLOC_MAX_BYTES:
        raise ValueError("more than one histogram run: not driven by this harness")
    if F % MAX_PER_RUN == 0:
        raise ValueError("field length a multiple of MAX_PER_RUN: the reference skips its last chunk")
    num_tasks = m * m
    if multi:
        tasks = np.array([(i, j + m) for i in range(m) for j in range(m)], np.int32)
    else:
        tasks = np.array([(i, j) for i in range(m) for j in range(m)], np.int32)
    bufs = []

    def alloc(nbytes):
        p = drv.alloc(nbytes)
        bufs.append(p)
        return p

    try:
        d_fields = alloc(rows * MAX_PER_RUN * 4)
        d_min = alloc(rows * 4)
        d_max = alloc(rows * 4)
        d_col = alloc(m * m * bins * 4)
        d_row = alloc(m * m * bins * 4)
        d_sim = alloc(m * m * 4)
        d_tasks = alloc(num_tasks * 8)
        d_joint = alloc(hist_bytes)
        drv.memset0(d_col, m * m * bins * 4)
        drv.memset0(d_row, m * m * bins * 4)
        drv.memset0(d_sim, m * m * 4)
        drv.memset0(d_joint, hist_bytes)
        drv.h2d(d_min, mins)
        drv.h2d(d_max, maxs)
        drv.h2d(d_tasks, tasks)
        # calculateRunInfo with one run: every ordered pair in it, histograms
        # indexed modulo their total size
        ri = RunInfo(tasksPerRun=num_tasks, lastRunMemBytes=hist_bytes, histMemMax=hist_bytes, offsetMax=1,
                     memoryPerRun=hist_bytes, odd=False, maxSize=hist_bytes // 4, fieldMaxMemory=0,
                     fieldsLastRun=False, fieldsLastRunBytes=0, multi=multi)
        di = DataInfo(F, bins, m, m)
        grid = (num_tasks + block - 1) // block
        for off in range(0, F, MAX_PER_RUN):
            count = MAX_PER_RUN
            if off + MAX_PER_RUN >= F:
                ri.fieldsLastRun = True
                ri.fieldsLastRunBytes = F % MAX_PER_RUN
                count = ri.fieldsLastRunBytes
            chunk = np.zeros((rows, MAX_PER_RUN), np.float32)
            chunk[:, :count] = fields[:, off:off + count]
            drv.h2d(d_fields, chunk)
            args = [C.c_uint64(d_fields), C.c_uint64(d_min), C.c_uint64(d_max), C.c_uint64(d_joint),
                    C.c_uint64(d_col), C.c_uint64(d_row), C.c_uint64(d_tasks), C.c_ulong(0), C.c_ulong(off),
                    C.c_uint64(d_sim), ri, di]
            drv.launch(grid, block, args)
        sim = np.zeros(m * m, np.float32)
        joint = np.zeros(m * m * bins * bins, np.uint32)
        col = np.zeros(m * m * bins, np.uint32)
        row = np.zeros(m * m * bins, np.uint32)
        drv.d2h(sim, d_sim)
        drv.d2h(joint, d_joint)
        drv.d2h(col, d_col)
        drv.d2h(row, d_row)
    finally:
        for p in bufs:
            drv.free(p)
    return sim.reshape(m, m), joint.reshape(m * m, bins, bins), col.reshape(m * m, bins), row.reshape(m * m, bins)


# ---------------------------------------------------------------------------
# Marching cubes: the reference's classifyVoxel, compactVoxels and
# generateTriangles (isosurfaces_cuda/src/MarchingCube.cu:84-124,138-149,
# 189-331), compiled from its sources by oracle/build_ref.sh into
# oracle/_ref/ref_mc.cubin together with oracle/ref_mc_wrap.cu.
MC_CUBIN = os.path.join(HERE, "_ref", "ref_mc.cubin")
MC_THREADS = 128                  # MarchingCube.cpp:591
MC_NTHREADS = 32                  # isosurfaces_cuda/src/defines.h (NTHREADS)
MC_CLASSIFY = b"_Z13classifyVoxelPjS_Pf5uint3f"
MC_COMPACT = b"_Z13compactVoxelsPjS_S_j"
MC_GENERATE = b"_Z17generateTrianglesP6float4S0_PjS1_Ph5uint3fjj"
MC_BIND = b"refshim_mc_bind"


class Uint3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


def mc_available():
    return os.path.exists(MC_CUBIN)


def _exclusive_scan_u32(a):
    """thrust::exclusive_scan over uint (thrustWrapper.cu ThrustScanWrapper):
    unsigned 32-bit sums."""
    out = np.zeros_like(a)
    c = np.cumsum(a.astype(np.uint64))
    out[1:] = (c[:-1] & 0xFFFFFFFF).astype(np.uint32)
    return out


def marching_cubes(volume, dims, iso):
    """The reference's cudaMarchingCube (MarchingCube.cpp:588-710) for one
    isovalue, with its own kernels on this GPU.  volume: the flat float32
    array the reference receives, dims = (dim.x, dim.y, dim.z) with x fastest
    in the kernels' indexing.  The host steps follow the reference's:
      * classify on the grid of :594-608 (V/128 blocks of 128, truncated,
        reshaped to 32768 x (V/128/32768) above 65535 blocks) -- voxels past
        that grid keep the zeros their buffers start with;
      * exclusive scans of the occupancy and vertex counts (thrust in the
        reference; here the same unsigned sums on the host), the active and
        total counts from the last elements (:624-636, :654-666);
      * compactVoxels on the classify grid, generateTriangles with NTHREADS
        threads on ceil(active/NTHREADS) blocks, halved in x and doubled in y
        while above 65535 (:668-694), maxVerts = V (Isosurface.cpp:263);
      * the first min(maxVerts, totalVerts) positions sorted and made unique
        (thrustWrapper.cu:44-56; lexicographic over x, y, z, w).
    Returns (unique xyz [n, 3] float32 in sorted order, active voxels, total
    vertices)."""
    drv = _driver()
    X, Y, Z = (int(d) for d in dims)
    V = X * Y * Z
    vol = np.ascontiguousarray(volume, np.float32).ravel()
    if vol.size != V:
        raise ValueError("volume size does not match dims")
    if V < MC_THREADS:
        raise ValueError("fewer voxels than one classify block: the reference launches an empty grid")
    fn = {k: drv.function(MC_CUBIN, k) for k in (MC_CLASSIFY, MC_COMPACT, MC_GENERATE, MC_BIND)}
    gx, gy = V // MC_THREADS, 1
    if gx > 65535:
        gy, gx = gx // 32768, 32768
    bufs = []

    def alloc(nbytes, zero=True):
        p = drv.alloc(nbytes)
        bufs.append(p)
        if zero:
            drv.memset0(p, nbytes)
        return p

    try:
        d_vol = alloc(V * 4, zero=False)
        drv.h2d(d_vol, vol)
        d_verts = alloc(V * 4)
        d_verts_scan = alloc(V * 4)
        d_occ = alloc(V * 4)
        d_occ_scan = alloc(V * 4)
        d_comp = alloc(V * 4)
        drv.launch(1, 1, [C.c_uint64(d_vol)], fn[MC_BIND])
        grid = Uint3(X, Y, Z)
        drv.launch((gx, gy), MC_THREADS,
                   [C.c_uint64(d_verts), C.c_uint64(d_occ), C.c_uint64(d_vol), grid, C.c_float(iso)],
                   fn[MC_CLASSIFY])
        occ = np.zeros(V, np.uint32)
        drv.d2h(occ, d_occ)
        occ_scan = _exclusive_scan_u32(occ)
        active = int(occ[-1]) + int(occ_scan[-1])
        if active == 0:
            return np.zeros((0, 3), np.float32), 0, 0
        drv.h2d(d_occ_scan, occ_scan)
        drv.launch((gx, gy), MC_THREADS,
                   [C.c_uint64(d_comp), C.c_uint64(d_occ), C.c_uint64(d_occ_scan), C.c_uint(V)], fn[MC_COMPACT])
        verts = np.zeros(V, np.uint32)
        drv.d2h(verts, d_verts)
        verts_scan = _exclusive_scan_u32(verts)
        total = int(verts[-1]) + int(verts_scan[-1])
        drv.h2d(d_verts_scan, verts_scan)
        g2x, g2y = -(-active // MC_NTHREADS), 1
        while g2x > 65535:
            g2x //= 2
            g2y *= 2
        max_verts = V
        d_pos = alloc(max_verts * 16)
        d_norm = alloc(max_verts * 16)
        drv.launch((g2x, g2y), MC_NTHREADS,
                   [C.c_uint64(d_pos), C.c_uint64(d_norm), C.c_uint64(d_comp), C.c_uint64(d_verts_scan),
                    C.c_uint64(d_vol), grid, C.c_float(iso), C.c_uint(active), C.c_uint(max_verts)],
                   fn[MC_GENERATE])
        n = min(max_verts, total)
        pos = np.zeros((n, 4), np.float32)
        if n:
            drv.d2h(pos, d_pos)
    finally:
        for p in bufs:
            drv.free(p)
    order = np.lexsort((pos[:, 3], pos[:, 2], pos[:, 1], pos[:, 0]))
    pos = pos[order]
    keep = np.ones(len(pos), bool)
    keep[1:] = np.any(pos[1:] != pos[:-1], axis=1)
    return np.ascontiguousarray(pos[keep, :3]), active, total
