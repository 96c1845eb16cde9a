/* Harness around the reference's own joint-histogram code
 * (isosurfaces_cuda/src/JointHistogram.cu), compiled from the reference sources
 * by oracle/build_ref.sh into oracle/_ref/.  TEST INFRASTRUCTURE: only the
 * checker and the CPU-baseline leg of bench.py load the result.
 *
 * The reference drives calculate_histogram_CPU with the same task list, run
 * info and 1M-voxel chunking as its GPU entry calculate_histogram_h
 * (JointHistogram.cu:266-420); ref_similarity_map_cpu repeats that host loop on
 * the CPU (field chunks are copied into the stride-MAX_PER_RUN staging buffer
 * exactly as the GPU entry copies them to the device). */
#include "isosurfaces_cuda/src/JointHistogram.cu"
#include <cfloat>
#include <cstdlib>
#include <cstring>
#include <thread>

extern "C" float ref_mutual_information(unsigned int *hist, int bins, float num_values,
                                        unsigned int *col_sums, unsigned int *row_sums)
{
    return calculateMutualInformation(hist, bins, bins, num_values, col_sums, row_sums);
}

extern "C" int ref_find_bucket(float val, float min_value, float step, int bins)
{
    return findBucket_d(val, min_value, step, bins, 0, 0);
}

/* fields: m arrays of length n (or 2m with multi).  Outputs: sim_map (m*m),
 * joint (m*m*H*H, may be NULL -> internal), col/row sums (m*m*H each, may be NULL).
 * threads > 1 splits the task list into contiguous runs, one per thread
 * (calculate_histogram_CPU's offset argument selects the run). */
extern "C" int ref_similarity_map_cpu(const float *const *fields, long n, int m, int bins, int multi,
                                      int threads, float *sim_map, unsigned int *joint_out,
                                      unsigned int *col_out, unsigned int *row_out)
{
    unsigned long nf = (unsigned long)m;
    unsigned long numTasks = nf * nf;
    int2 *tasks = (int2 *)malloc(sizeof(int2) * numTasks);
    size_t c = 0;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) tasks[c++] = make_int2(i, multi ? j + m : j);
    unsigned long histWords = numTasks * (unsigned long)bins * bins;
    unsigned int *joint = joint_out ? joint_out : (unsigned int *)malloc(sizeof(unsigned int) * histWords);
    unsigned int *cols = col_out ? col_out : (unsigned int *)malloc(sizeof(unsigned int) * numTasks * bins);
    unsigned int *rows = row_out ? row_out : (unsigned int *)malloc(sizeof(unsigned int) * numTasks * bins);
    memset(joint, 0, sizeof(unsigned int) * histWords);
    memset(cols, 0, sizeof(unsigned int) * numTasks * bins);
    memset(rows, 0, sizeof(unsigned int) * numTasks * bins);
    int nfields = m * (multi ? 2 : 1);
    float *mins = (float *)malloc(sizeof(float) * nfields);
    float *maxs = (float *)malloc(sizeof(float) * nfields);
    for (int k = 0; k < nfields; ++k) {
        float mn = FLT_MAX, mx = FLT_MIN;   /* DistanceField::getInterval */
        for (long v = 0; v < n; ++v) { float x = fields[k][v]; if (x < mn) mn = x; if (x > mx) mx = x; }
        mins[k] = mn; maxs[k] = mx;
    }
    float *staging = (float *)malloc(sizeof(float) * (size_t)nfields * MAX_PER_RUN);
    if (threads < 1) threads = 1;
    if ((unsigned long)threads > numTasks) threads = (int)numTasks;
    unsigned long perThread = (numTasks + threads - 1) / threads;
    dataInfo dInfo = {(int)n, bins, m, m};
    for (unsigned long fieldOffset = 0; fieldOffset < (unsigned long)n; fieldOffset += MAX_PER_RUN) {
        runInfo rInfo;
        memset(&rInfo, 0, sizeof rInfo);
        rInfo.tasksPerRun = perThread;
        rInfo.offsetMax = (numTasks + perThread - 1) / perThread;
        rInfo.maxSize = histWords;
        rInfo.multi = multi != 0;
        unsigned long count = MAX_PER_RUN;
        if (fieldOffset + MAX_PER_RUN >= (unsigned long)n) {
            rInfo.fieldsLastRun = true;
            rInfo.fieldsLastRunBytes = (unsigned long)(n % MAX_PER_RUN);
            count = rInfo.fieldsLastRunBytes;
        }
        for (int k = 0; k < nfields; ++k)
            memcpy(&staging[(size_t)k * MAX_PER_RUN], &fields[k][fieldOffset], sizeof(float) * count);
        std::thread *pool = new std::thread[threads];
        for (int t = 0; t < threads; ++t) {
            pool[t] = std::thread([=]() {
                runInfo r = rInfo;
                /* the last run may hold fewer tasks: trim tasksPerRun for it */
                unsigned long first = (unsigned long)t * perThread;
                if (first >= numTasks) return;
                if (first + r.tasksPerRun > numTasks) r.tasksPerRun = numTasks - first;
                /* the task pointer is shifted to this thread's run; offset stays 0 */
                calculate_histogram_CPU(staging, mins, maxs, joint, cols, rows, tasks + first, 0, 0,
                                        sim_map, r, dInfo);
            });
        }
        for (int t = 0; t < threads; ++t) pool[t].join();
        delete[] pool;
    }
    free(staging); free(mins); free(maxs); free(tasks);
    if (!joint_out) free(joint);
    if (!col_out) free(cols);
    if (!row_out) free(rows);
    return 0;
}
