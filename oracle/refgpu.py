"""The reference's own GPU histogram kernel, run on this machine's GPU (test
infrastructure only: a checker, never the engine).

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
        mod = C.c_void_p()
        self._check(cu.cuModuleLoad(C.byref(mod), CUBIN.encode()), "cuModuleLoad")
        fn = C.c_void_p()
        self._check(cu.cuModuleGetFunction(C.byref(fn), mod, KERNEL), "cuModuleGetFunction")
        self.fn = fn
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

    def launch(self, grid, block, args):
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn, grid, 1, 1, block, 1, 1, 0, None, ptrs, None), "cuLaunchKernel")
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


_DRIVER = None


def similarity(fields, bins, mins=None, maxs=None, multi=False, block=128):
    """The reference's calculate_histogram_h on the GPU for m fields (2m rows
    in multi mode: the first m against the last m).  fields: [rows, F]
    float32.  mins/maxs: per-row interval (default: each row's min and max,
    the values DistanceField::getInterval gives for non-negative fields).
    Returns (sim [m, m] float32, joint [m*m, bins, bins] uint32,
    col_sums [m*m, bins], row_sums [m*m, bins])."""
    global _DRIVER
    if _DRIVER is None:
        _DRIVER = _Driver()
    drv = _DRIVER
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
