"""The GPU checker's restatements of the reference's host-side launch
arithmetic, on the CPU: calculateRunInfo's histogram runs
(JointHistogram.cu:231-264) and the coverage of generateTriangles' halved
grid (MarchingCube.cpp:668-678)."""
import refgpu


def hist_bytes(m, bins=256):
    return m * m * bins * bins * 4


def test_single_run():
    m = 64
    tpr, last, hmax, runs, per_run, odd = refgpu.run_info(m * m, hist_bytes(m), m * m)
    assert (tpr, runs, odd) == (4096, 1, False)
    assert per_run == hmax == last == hist_bytes(m)


def test_even_pair_count_two_runs():
    m = 96
    tpr, last, hmax, runs, per_run, odd = refgpu.run_info(m * m, hist_bytes(m), m * m)
    assert (tpr, runs, odd) == (4608, 2, False)
    assert per_run == tpr * 256 * 256 * 4


def test_odd_pair_count_adds_a_one_pair_run():
    m = 91
    tpr, last, hmax, runs, per_run, odd = refgpu.run_info(m * m, hist_bytes(m), m * m)
    assert (tpr, runs, odd) == (4140, 3, True)
    assert last == 256 * 256 * 4                  # the last run holds one histogram
    assert per_run == tpr * 256 * 256 * 4         # runs of tasksPerRun histograms, no aliasing


def test_benchmark_map_runs_are_powers_of_two():
    m = 256
    tpr, _, _, runs, per_run, _ = refgpu.run_info(m * m, hist_bytes(m), m * m)
    assert (tpr, runs) == (8192, 8)
    size = per_run // 4
    assert size & (size - 1) == 0                 # the wrapped 32-bit index stays harmless


def test_generated_voxels():
    assert refgpu.mc_generated_voxels(1000) == 1000
    assert refgpu.mc_generated_voxels(65535 * 32) == 65535 * 32
    # 3,611,220 active voxels: 112,851 blocks -> 56,425 x 2 after one halving
    assert refgpu.mc_generated_voxels(3611220) == 56425 * 2 * 32
