"""The reference's own GPU kernels -- its joint histogram, marching cubes,
LBVH and voxel approximation -- run on this machine's GPU (test
infrastructure only: a checker, never the engine).  The histogram harness is
similarity(); marching_cubes(), lbvh_distance_field() and approximation()
follow below.

oracle/build_ref.sh compiles isosurfaces_cuda/src/JointHistogram.cu from the
reference's sources, device code only and with nvcc's default flags (as the
reference's CMake build passes none), into oracle/_ref/ref_histogram.cubin.
This module loads that cubin through the CUDA driver API (ctypes on
libcuda.so.1) and drives its kernel calculate_histogram_g (JointHistogram.cu:
100-162) the way the reference's host function calculate_histogram_h
(JointHistogram.cu:266-420) does:

  * one task per ordered pair, (i, j) for i, j < m in row-major order, or
    (i, j + m) in multi mode (:306-328);
  * fields staged in chunks of MAX_PER_RUN = 1,000,000 values at stride
    MAX_PER_RUN (:377-392), one kernel launch per chunk, the last chunk
    flagged so the kernel evaluates calculateMutualInformation (:156-160);
  * the runs of calculateRunInfo (:231-264): as many as the m*m histograms
    need at MALLOC_MAX_BYTES (2 GiB, isosurfaces_cuda/hdr/common.h:8) per
    allocation, each over every field chunk.

The result is the reference's own output on the GPU: its FP32 similarity map
(every ordered pair), its column and row sums, and its joint histograms when
the map takes one run.
Sizes whose last chunk would be empty (the reference's loop skips a chunk
when the field length is a multiple of MAX_PER_RUN), and sizes where the
kernel's 32-bit histogram index overflows onto other pairs' histograms, are
refused here rather than run.
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
        self.fn = self.function(CUBIN, KERNEL) if os.path.exists(CUBIN) else None
        self.ev0, self.ev1 = C.c_void_p(), C.c_void_p()
        self._check(cu.cuEventCreate(C.byref(self.ev0), 0), "cuEventCreate")
        self._check(cu.cuEventCreate(C.byref(self.ev1), 0), "cuEventCreate")
        cu.cuMemAlloc_v2.argtypes = [C.POINTER(C.c_uint64), C.c_size_t]
        cu.cuMemFree_v2.argtypes = [C.c_uint64]
        cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        cu.cuMemcpyDtoH_v2.argtypes = [C.c_void_p, C.c_uint64, C.c_size_t]
        cu.cuMemsetD8_v2.argtypes = [C.c_uint64, C.c_ubyte, C.c_size_t]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]
        cu.cuEventRecord.argtypes = [C.c_void_p, C.c_void_p]
        cu.cuEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]

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

    def memset0(self, p, nbytes, value=0):
        self._check(self.cu.cuMemsetD8_v2(p, value, nbytes), "cuMemsetD8")

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
        """grid: an int (x) or an (x, y) pair; one synchronising launch.
        Returns the launch's device time in ms (CUDA events around it)."""
        gx, gy = (grid, 1) if isinstance(grid, int) else grid
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuEventRecord(self.ev0, None), "cuEventRecord")
        self._check(self.cu.cuLaunchKernel(fn if fn is not None else self.fn, gx, gy, 1, block, 1, 1, 0, None,
                                           ptrs, None), "cuLaunchKernel")
        self._check(self.cu.cuEventRecord(self.ev1, None), "cuEventRecord")
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")
        ms = C.c_float()
        self._check(self.cu.cuEventElapsedTime(C.byref(ms), self.ev0, self.ev1), "cuEventElapsedTime")
        return ms.value


_DRIVER = None


def _driver():
    global _DRIVER
    if _DRIVER is None:
        _DRIVER = _Driver()
    return _DRIVER


def _account(timing, name, ms):
    if timing is not None:
        timing[name] = timing.get(name, 0.0) + ms


def run_info(num_tasks, hist_bytes, num_hist):
    """calculateRunInfo (JointHistogram.cu:231-264), integer for integer:
    (tasksPerRun, lastRunMemBytes, histMemMax, offsetMax, memoryPerRun, odd).
    offsetMax runs of tasksPerRun tasks share one allocation of memoryPerRun
    bytes; with an odd task count over several runs, one more run takes the
    last task alone."""
    offset_max, hist_mem_max = 1, hist_bytes
    if hist_bytes > MALLOC_MAX_BYTES:
        offset_max = 2
        while offset_max * MALLOC_MAX_BYTES < hist_bytes:
            offset_max += 1
        hist_mem_max = hist_bytes // offset_max
    last_run = hist_mem_max
    tasks_per_run = num_tasks // offset_max
    odd = num_tasks % 2 == 1 and offset_max > 1
    mem_per_run = hist_mem_max
    mem_per_hist = hist_bytes // num_hist
    if odd:
        mem_per_run = hist_mem_max - mem_per_hist // offset_max
        offset_max += 1
        last_run = mem_per_hist
    return tasks_per_run, last_run, hist_mem_max, offset_max, mem_per_run, odd


def similarity(fields, bins, mins=None, maxs=None, multi=False, block=128, timing=None):
    """The reference's calculate_histogram_h on the GPU for m fields (2m rows
    in multi mode: the first m against the last m).  fields: [rows, F]
    float32.  mins/maxs: per-row interval (default: each row's min and max,
    the values DistanceField::getInterval gives for non-negative fields).
    Runs as many histogram runs as calculateRunInfo gives, each over every
    1,000,000-value chunk of the fields (JointHistogram.cu:372-392).
    Returns (sim [m, m] float32, joint [m*m, bins, bins] uint32 or None when
    the map takes several runs (the reference keeps only one run's histograms
    at a time), col_sums [m*m, bins], row_sums [m*m, bins]).  timing (a
    dict), if given, accumulates the device ms of each kernel by name."""
    drv = _driver()
    fields = np.ascontiguousarray(fields, dtype=np.float32)
    rows, F = fields.shape
    m = rows // 2 if multi else rows
    if mins is None:
        mins = fields.min(axis=1)
        maxs = fields.max(axis=1)
    mins = np.ascontiguousarray(mins, np.float32)
    maxs = np.ascontiguousarray(maxs, np.float32)
    if F % MAX_PER_RUN == 0:
        raise ValueError("field length a multiple of MAX_PER_RUN: the reference skips its last chunk")
    num_tasks = m * m
    hist_bytes = num_tasks * bins * bins * 4
    max_size = run_info(num_tasks, hist_bytes, num_tasks)[4] // 4
    if num_tasks * bins * bins > 2 ** 31 and max_size & (max_size - 1):
        # the kernel's histogram index (id1 * m + id2) * bins^2 + bin is a
        # 32-bit int (JointHistogram.cu:133-135, :151); once it wraps, its
        # value modulo a run size that is not a power of two lands in other
        # pairs' histograms
        raise ValueError("the reference's 32-bit histogram index wraps onto other pairs' histograms here")
    if multi:
        tasks = np.array([(i, j + m) for i in range(m) for j in range(m)], np.int32)
    else:
        tasks = np.array([(i, j) for i in range(m) for j in range(m)], np.int32)
    tasks_per_run, last_run, hist_mem_max, offset_max, mem_per_run, odd = run_info(num_tasks, hist_bytes, num_tasks)
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
        d_joint = alloc(mem_per_run)
        drv.memset0(d_col, m * m * bins * 4)
        drv.memset0(d_row, m * m * bins * 4)
        drv.memset0(d_sim, m * m * 4)
        drv.h2d(d_min, mins)
        drv.h2d(d_max, maxs)
        drv.h2d(d_tasks, tasks)
        ri = RunInfo(tasksPerRun=tasks_per_run, lastRunMemBytes=last_run, histMemMax=hist_mem_max,
                     offsetMax=offset_max, memoryPerRun=mem_per_run, odd=odd, maxSize=mem_per_run // 4,
                     fieldMaxMemory=0, fieldsLastRun=False, fieldsLastRunBytes=0, multi=multi)
        di = DataInfo(F, bins, m, m)
        grid = (tasks_per_run + block - 1) // block
        chunk = np.zeros((rows, MAX_PER_RUN), np.float32)
        for run in range(offset_max):
            drv.memset0(d_joint, mem_per_run)
            ri.fieldsLastRun = False
            for off in range(0, F, MAX_PER_RUN):
                count = MAX_PER_RUN
                if off + MAX_PER_RUN >= F:
                    ri.fieldsLastRun = True
                    ri.fieldsLastRunBytes = F % MAX_PER_RUN
                    count = ri.fieldsLastRunBytes
                chunk[:] = 0
                chunk[:, :count] = fields[:, off:off + count]
                drv.h2d(d_fields, chunk)
                args = [C.c_uint64(d_fields), C.c_uint64(d_min), C.c_uint64(d_max), C.c_uint64(d_joint),
                        C.c_uint64(d_col), C.c_uint64(d_row), C.c_uint64(d_tasks), C.c_ulong(run), C.c_ulong(off),
                        C.c_uint64(d_sim), ri, di]
                _account(timing, "calculate_histogram_g", drv.launch(grid, block, args))
        sim = np.zeros(m * m, np.float32)
        col = np.zeros(m * m * bins, np.uint32)
        row = np.zeros(m * m * bins, np.uint32)
        drv.d2h(sim, d_sim)
        drv.d2h(col, d_col)
        drv.d2h(row, d_row)
        joint = None
        if offset_max == 1:
            joint = np.zeros(m * m * bins * bins, np.uint32)
            drv.d2h(joint, d_joint)
            joint = joint.reshape(m * m, bins, bins)
    finally:
        for p in bufs:
            drv.free(p)
    return sim.reshape(m, m), joint, col.reshape(m * m, bins), row.reshape(m * m, bins)


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


def mc_generated_voxels(active):
    """Active voxels the reference's generateTriangles launch covers: NTHREADS
    per block on ceil(active / NTHREADS) blocks, halved in x (rounding down)
    and doubled in y while above 65535 (MarchingCube.cpp:668-678), so an odd
    count loses blocks."""
    gx, gy = -(-int(active) // MC_NTHREADS), 1
    while gx > 65535:
        gx //= 2
        gy *= 2
    return min(int(active), gx * gy * MC_NTHREADS)


def marching_cubes(volume, dims, iso, with_w=False, timing=None):
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
    vertices); with with_w, the rows keep their w, which is 1 for every
    position the kernel wrote and 0 for the zeros of entries it left unwritten
    (more than maxVerts - 3 triangle vertices, MarchingCube.cu:319) or
    did not reach (voxels past mc_generated_voxels).  timing (a dict), if
    given, accumulates the device ms of each of the reference's kernels."""
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
        _account(timing, "classifyVoxel", drv.launch(
            (gx, gy), MC_THREADS, [C.c_uint64(d_verts), C.c_uint64(d_occ), C.c_uint64(d_vol), grid, C.c_float(iso)],
            fn[MC_CLASSIFY]))
        occ = np.zeros(V, np.uint32)
        drv.d2h(occ, d_occ)
        occ_scan = _exclusive_scan_u32(occ)
        active = int(occ[-1]) + int(occ_scan[-1])
        if active == 0:
            return np.zeros((0, 4 if with_w else 3), np.float32), 0, 0
        drv.h2d(d_occ_scan, occ_scan)
        _account(timing, "compactVoxels", drv.launch(
            (gx, gy), MC_THREADS, [C.c_uint64(d_comp), C.c_uint64(d_occ), C.c_uint64(d_occ_scan), C.c_uint(V)],
            fn[MC_COMPACT]))
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
        _account(timing, "generateTriangles", drv.launch(
            (g2x, g2y), MC_NTHREADS,
            [C.c_uint64(d_pos), C.c_uint64(d_norm), C.c_uint64(d_comp), C.c_uint64(d_verts_scan), C.c_uint64(d_vol),
             grid, C.c_float(iso), C.c_uint(active), C.c_uint(max_verts)], fn[MC_GENERATE]))
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
    return np.ascontiguousarray(pos[keep] if with_w else pos[keep, :3]), active, total


# ---------------------------------------------------------------------------
# LBVH distance fields: the reference's calculateMortonCodes_g, initLeaves_g,
# initNodes_g, generateInternalNodes_g, createBoundingVolumes_g and
# traverseTree_g (isosurfaces_cuda/src/BVH.cu:108-118,247-368,577-613),
# compiled from its sources by oracle/build_ref.sh into oracle/_ref/ref_bvh.cubin
# together with oracle/ref_bvh_wrap.cu.
BVH_CUBIN = os.path.join(HERE, "_ref", "ref_bvh.cubin")
BVH_THREADS = 256
BVH_NUM_SAMPLES = 1500            # runtime/hdr/globals.h (NUM_SAMPLES)
BVH_MAX_DEPTH = 60                # traverseIterative_d keeps a 64-entry stack (BVH.cu:515)
BVH_MORTON = b"_Z22calculateMortonCodes_gP6float3iPj"
BVH_LEAVES = b"_Z12initLeaves_gP8LeafNodeP6float3Pji"
BVH_NODES = b"_Z11initNodes_gP12InternalNodei"
BVH_BUILD = b"_Z23generateInternalNodes_gP8LeafNodeP12InternalNodePjii"
BVH_BOXES = b"_Z23createBoundingVolumes_gP8LeafNodeP12InternalNodePii"
BVH_TRAVERSE = b"_Z14traverseTree_gP8LeafNodeP12InternalNodePfiiiiiiPjiP6float3b"
BVH_SIZES = b"refshim_bvh_sizes"


def bvh_available():
    return os.path.exists(BVH_CUBIN)


def _blocks(n, threads):
    return (int(n) + threads - 1) // threads


def lbvh_distance_field(points, dims, ds=1, num_samples=BVH_NUM_SAMPLES, timing=None):
    """The reference's generateHierarchy_h (BVH.cu:815-875) for one surface,
    with its own kernels on this GPU.  points: [P, 3] float32, already divided
    by the largest dimension as generateHierarchy_W does (funcs.cpp:150-160);
    dims = the volume's (dimX, dimY, dimZ).  Returns the float32 field of
    (dimX/ds)(dimY/ds)(dimZ/ds) samples in the reference's order.

    The reference's kernels are run only on a tree that has been checked
    first: the Morton codes from its kernel must equal the restatement's
    (oracle.ref_morton); the codes are sorted on the host by a stable sort (as
    thrust's radix sort_by_key orders equal keys); the restated tree
    (oracle.ref_lbvh) must be a tree no deeper than BVH_MAX_DEPTH; and the
    child ids the reference's build kernel writes must equal the restated
    ones before the box and traversal kernels run.  The seeds of the
    traversal are the reference's (traverse_h, BVH.cu:640-644: unsigned
    32-bit i * P / numSamples).  timing (a dict), if given, accumulates the
    device ms of each of the reference's kernels."""
    import oracle
    drv = _driver()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = pts.shape[0]
    if n < 2:
        raise ValueError("fewer than two points: the reference launches empty grids")
    X, Y, Z = (int(d) for d in dims)
    size = (X // ds) * (Y // ds) * (Z // ds)
    fn = {k: drv.function(BVH_CUBIN, k) for k in
          (BVH_MORTON, BVH_LEAVES, BVH_NODES, BVH_BUILD, BVH_BOXES, BVH_TRAVERSE, BVH_SIZES)}
    bufs = []

    def alloc(nbytes, zero=True):
        p = drv.alloc(nbytes)
        bufs.append(p)
        if zero:
            drv.memset0(p, nbytes)
        return p

    try:
        d_info = alloc(64)
        drv.launch(1, 1, [C.c_uint64(d_info)], fn[BVH_SIZES])
        info = np.zeros(16, np.int32)
        drv.d2h(info, d_info)
        leaf_sz, node_sz, f3_sz, off_l, off_r = (int(v) for v in info[:5])
        if f3_sz != 12:
            raise RuntimeError("unexpected float3 size %d" % f3_sz)
        d_pts = alloc(n * 12, zero=False)
        d_codes = alloc(n * 4)
        drv.h2d(d_pts, pts)
        _account(timing, "calculateMortonCodes_g", drv.launch(
            _blocks(n, BVH_THREADS), BVH_THREADS, [C.c_uint64(d_pts), C.c_int(n), C.c_uint64(d_codes)],
            fn[BVH_MORTON]))
        codes = np.zeros(n, np.uint32)
        drv.d2h(codes, d_codes)
        if not np.array_equal(codes, oracle.ref_morton(pts)):
            raise RuntimeError("the reference's Morton codes differ from the restatement: tree not built")
        order = np.argsort(codes, kind="stable")
        codes = np.ascontiguousarray(codes[order])
        drv.h2d(d_codes, codes)
        drv.h2d(d_pts, np.ascontiguousarray(pts[order]))
        left, right, depth = oracle.ref_lbvh(codes)
        if depth < 0 or depth > BVH_MAX_DEPTH:
            raise ValueError("the reference's rules give no tree of depth <= %d here (%d): not run"
                             % (BVH_MAX_DEPTH, depth))
        d_leaves = alloc(n * leaf_sz)
        d_nodes = alloc((n - 1) * node_sz)
        _account(timing, "initLeaves_g", drv.launch(
            _blocks(n, BVH_THREADS), BVH_THREADS,
            [C.c_uint64(d_leaves), C.c_uint64(d_pts), C.c_uint64(d_codes), C.c_int(n)], fn[BVH_LEAVES]))
        _account(timing, "initNodes_g", drv.launch(
            _blocks(n - 1, BVH_THREADS), BVH_THREADS, [C.c_uint64(d_nodes), C.c_int(n - 1)], fn[BVH_NODES]))
        _account(timing, "generateInternalNodes_g", drv.launch(
            _blocks(n - 1, BVH_THREADS), BVH_THREADS,
            [C.c_uint64(d_leaves), C.c_uint64(d_nodes), C.c_uint64(d_codes), C.c_int(n), C.c_int(n - 1)],
            fn[BVH_BUILD]))
        raw = np.zeros((n - 1) * node_sz, np.uint8)
        drv.d2h(raw, d_nodes)
        raw = raw.reshape(n - 1, node_sz)
        gl = raw[:, off_l:off_l + 4].copy().view(np.int32).ravel()
        gr = raw[:, off_r:off_r + 4].copy().view(np.int32).ravel()
        if not (np.array_equal(gl, left) and np.array_equal(gr, right)):
            raise RuntimeError("the reference's build kernel made another tree than the checked one: not traversed")
        d_block = alloc(n * 4)
        _account(timing, "createBoundingVolumes_g", drv.launch(
            _blocks(n, BVH_THREADS), BVH_THREADS,
            [C.c_uint64(d_leaves), C.c_uint64(d_nodes), C.c_uint64(d_block), C.c_int(n)], fn[BVH_BOXES]))
        ns = min(int(num_samples), n)
        ids = ((np.arange(ns, dtype=np.uint64) * np.uint64(n)) & np.uint64(0xFFFFFFFF)) // np.uint64(ns)
        ids = ids.astype(np.uint32)
        if ids.max() >= n:
            raise RuntimeError("seed index out of range")
        d_ids = alloc(ns * 4)
        drv.h2d(d_ids, ids)
        d_dist = alloc(size * 4)
        _account(timing, "traverseTree_g", drv.launch(
            _blocks(size, BVH_THREADS), BVH_THREADS,
            [C.c_uint64(d_leaves), C.c_uint64(d_nodes), C.c_uint64(d_dist), C.c_int(size), C.c_int(X), C.c_int(Y),
             C.c_int(Z), C.c_int(ns), C.c_int(n), C.c_uint64(d_ids), C.c_int(ds), C.c_uint64(0), C.c_bool(False)],
            fn[BVH_TRAVERSE]))
        out = np.zeros(size, np.float32)
        drv.d2h(out, d_dist)
    finally:
        for p in bufs:
            drv.free(p)
    return out



# ---------------------------------------------------------------------------
# Voxel approximation: the reference's calculate_approximation_g
# (isosurfaces_cuda/src/IsosurfaceApproximation.cu:120-135), compiled from its
# sources by oracle/build_ref.sh into oracle/_ref/ref_approx.cubin.
APPROX_CUBIN = os.path.join(HERE, "_ref", "ref_approx.cubin")
APPROX_KERNEL = b"_Z25calculate_approximation_gPffiiiP4int3iii"
APPROX_THREADS = 256              # IsosurfaceApproximation.cu:162
APPROX_MAX_BLOCKS = 2 << 14       # :163


def approx_available():
    return os.path.exists(APPROX_CUBIN)


def approximation(volume, dims, iso, timing=None):
    """The reference's approximate_isosurfaces_h (IsosurfaceApproximation.cu:
    159-208) at scale 1 with its own kernel on this GPU: the cell array set to
    all-ones bytes, launches of 32,768 blocks of 256 threads at block offsets
    0, 32768, ... until the volume is covered, then the stable compaction of
    the cells whose x is not negative (thrust::copy_if with is_positive,
    thrustWrapper.h:47-54; here on the host).  volume: X*Y*Z float32 with z
    fastest.  Returns the crossing cells as int32 [k, 3] in linear order."""
    drv = _driver()
    X, Y, Z = (int(d) for d in dims)
    V = X * Y * Z
    vol = np.ascontiguousarray(volume, np.float32).ravel()
    if vol.size != V or min(X, Y, Z) < 2:
        raise ValueError("volume size does not match dims, or a dimension below 2")
    num_cells = (X - 1) * (Y - 1) * (Z - 1)
    fn = drv.function(APPROX_CUBIN, APPROX_KERNEL)
    bufs = []
    try:
        d_vol = drv.alloc(V * 4)
        bufs.append(d_vol)
        d_cells = drv.alloc(num_cells * 12)
        bufs.append(d_cells)
        drv.h2d(d_vol, vol)
        drv.memset0(d_cells, num_cells * 12, 0xFF)
        blocks = (V + APPROX_THREADS - 1) // APPROX_THREADS
        for off in range(0, blocks, APPROX_MAX_BLOCKS):
            _account(timing, "calculate_approximation_g", drv.launch(
                APPROX_MAX_BLOCKS, APPROX_THREADS,
                [C.c_uint64(d_vol), C.c_float(iso), C.c_int(X), C.c_int(Y), C.c_int(Z), C.c_uint64(d_cells),
                 C.c_int(V), C.c_int(off), C.c_int(1)], fn))
        cells = np.zeros((num_cells, 3), np.int32)
        drv.d2h(cells, d_cells)
    finally:
        for p in bufs:
            drv.free(p)
    return np.ascontiguousarray(cells[cells[:, 0] >= 0])
