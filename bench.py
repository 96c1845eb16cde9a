"""Benchmark: ISM pairs per second of the isosurface-similarity pipeline.

One step = one isosurface similarity map of one volume: marching-cubes
surfaces for every isovalue, LBVH distance fields of the non-empty ones, joint
histograms of all unordered field pairs and FP64 NMI.  The default workload is
256^3 float32 (12 Gaussian blobs plus 0.05 k^-2 noise, seeded), 256 isovalues
inside the value range, 256 histogram bins: n(n-1)/2 = 32640 ISM pairs per
step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config 1|2|3] [--df lbvh|brute]

Under torchrun each rank computes its own replica (the pipeline shards by
volume; no collective on the data path) and rank 0 prints one JSON line.
--impl reference times the reference's histogram/NMI arithmetic and a CPU
restatement of its surface and distance stages on the host cores; beside that
value its line carries reference_gpu, the device time of the reference's own
kernels (compiled from its sources) on the same GPU, over a bounded sample.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "isosurface-analysis_gb300")
sys.path.insert(0, PKG)

METRIC = "ISM pairs/sec (256-isovalue ISM of a 256^3 volume, 256 bins)"


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_synth():
    """The synthetic-volume generators, loaded from their file: importing the
    isosim package would load the engine's library, which the reference arm
    must not have in its process."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("iso_bench_synth", os.path.join(PKG, "isosim", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload(config):
    synth = load_synth()
    if config == 1:
        vol, isos, bins = synth.config1()
        name = "64^3 8-blob volume, 32 isovalues, 128 bins"
    elif config == 2:
        vol, isos, bins = synth.config2()
        name = "128^3 k^-3 random field, 100 isovalues in [-2.5,2.5], 256 bins"
    else:
        vol, isos, bins = synth.config3()
        name = "256^3 12-blob + 0.05 k^-2 noise volume, 256 isovalues, 256 bins"
    return vol, isos, bins, name


def bench_config(args, name, n, bins, world):
    """The workload description both arms print (identical for equal flags)."""
    return {"workload": name, "isovalues": int(n), "bins": int(bins), "pairs_per_ism": int(n * (n - 1) // 2),
            "l2": "256 MB flush before every timed step",
            "parallelism": "replicas" if world > 1 else "single GPU"}


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sms)) if sms else None,
                "sm_max_mhz": float(max(maxs)) if maxs else None,
                "reasons": sorted(reasons), "samples": len(sms)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_BACKEND", "nccl") == "nccl" else "gloo")
        pg = dist
    return world, rank, local, pg


def max_over_ranks(pg, value):
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def run_ours(args):
    import torch

    import isosim

    world, rank, local, pg = dist_init()
    torch.cuda.set_device(local)
    vol, isos, bins, name = workload(args.config)
    X, Y, Z = vol.shape
    method = {"lbvh": isosim.DF_LBVH, "brute": isosim.DF_BRUTE, "tc": isosim.DF_TC}[args.df]
    ctx = isosim.Context(local)
    if getattr(args, "hist_seg", None) is not None:
        ctx.set_hist_segment_values(args.hist_seg)
    if args.hist_codes is not None:
        ctx.set_hist_row_codes(args.hist_codes)
    stream = torch.cuda.ExternalStream(ctx.stream)
    d_vol = torch.from_numpy(vol.ravel()).to(f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    n = len(isos)
    ism_dev = torch.empty(n * n, dtype=torch.float32, device=f"cuda:{local}")

    def step(vol_arg, out):
        return ctx.ism(vol_arg, (X, Y, Z), isos, surface=isosim.SURFACE_MC, frame=isosim.FRAME_REF,
                       df_method=method, bins=bins, out=out)

    # the engine's autotuner picks the launch shapes for this workload (cached
    # on disk; trials run before the warm-up, outside every timed region)
    tuning = None
    if not args.no_tune and args.hist_seg is None:
        import tempfile
        t = ctx.autotune(d_vol, (X, Y, Z), isos, surface=isosim.SURFACE_MC, frame=isosim.FRAME_REF,
                         df_method=method, bins=bins,
                         cache_path=os.path.join(tempfile.gettempdir(), "isosim_tune_cache.txt"))
        tuning = {"hist_segment_values": int(t.hist_segment_values), "lbvh_group_points": int(t.lbvh_group_points),
                  "query_run": int(t.query_run) or "by volume size", "from_cache": bool(t.from_cache),
                  "trials": int(t.trials), "default_ms": round(t.default_ms, 2), "tuned_ms": round(t.tuned_ms, 2)}
    # the ISM's MI evaluation: the reference's own FP32 evaluation (bit for bit
    # its kernel's map; the default) or the engine's FP64 NMI
    ctx.set_mi_mode(isosim.MI_REF32 if args.mi == "ref32" else isosim.MI_FP64)
    for _ in range(args.warmup):
        _, ids, sstats, timing = step(d_vol, ism_dev)
    m = len(ids)
    P = int(sum(sstats[k].points for k in range(len(isos))))  # surface points of all isovalues
    pairs = m * (m - 1) // 2
    torch.cuda.synchronize()

    # ---- device-resident throughput: CUDA events on the engine's stream, L2
    # flushed (256 MB write) before every step outside the timed interval
    sampler = ClockSampler(local)
    sampler.start()
    barrier(pg)
    torch.cuda.synchronize()
    launches0 = ctx.launches
    total_ms = 0.0
    stage = np.zeros(3)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        _, _, _, timing = step(d_vol, ism_dev)
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
        stage += [timing.surface_ms, timing.distance_ms, timing.histogram_ms]
    torch.cuda.synchronize()
    barrier(pg)
    launches = ctx.launches - launches0
    clocks = sampler.stop()
    t_step = max_over_ranks(pg, total_ms / args.steps)
    value = world * pairs / (t_step / 1e3)
    stage /= args.steps

    # ---- end to end through the C ABI with host buffers: pinned volume in,
    # ISM out to host memory, copies inside the timed region
    pinned = torch.from_numpy(vol.ravel()).pin_memory()
    host_out = np.zeros(n * n, dtype=np.float32)
    e2e_ms = 0.0
    for _ in range(max(1, min(args.steps, 3))):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step(pinned, host_out)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_ms /= max(1, min(args.steps, 3))
    e2e_ms = max_over_ranks(pg, e2e_ms)

    # ---- roofline of the histogram/NMI kernel (the O(n^2 V) stage): unique
    # bytes = each distance field read once + each joint histogram written once
    F = X * Y * Z
    hist_bytes = 4.0 * F * m + 4.0 * bins * bins * pairs
    seg_values = (tuning["hist_segment_values"] if tuning else
                  (2097152 if args.hist_seg is None else args.hist_seg))  # the engine's default
    hist_s = stage[2] / 1e3
    peak, peak_kind = load_peaks()
    achieved = hist_bytes / hist_s / 1e9
    counter_peak = ctx.counter_rate(bins if bins & (bins - 1) == 0 else 256)
    updates = F * pairs / hist_s
    # DRAM traffic of the histogram stage: --hist-traffic, else the committed
    # ncu summary of this workload when it was captured on the current
    # histogram source; otherwise null
    traffic, traffic_src = args.hist_traffic, "--hist-traffic"
    if traffic is None and args.config == 3 and bins == 256 and seg_values == 2097152 and args.mi == "ref32":
        traffic, traffic_src = histogram_traffic()
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic,
                "traffic_source": traffic_src,
                "traffic_over_unique": round(traffic / hist_bytes, 1) if traffic else None,
                "kernel": ("joint_histogram_wide_kernel" if bins <= 224 else
                           ("joint_histogram_seg_kernel + joint_mi_kernel" if 0 < seg_values < F
                            else "joint_histogram_mi_kernel")) + (" + mi_ref32_kernel" if args.mi == "ref32" else ""),
                "peak_source": peak_kind,
                "note": "unique bytes (each field read once, one bins^2 histogram per pair); the kernel is "
                        "bound by its counter updates: see smem_atomic",
                "smem_atomic": {"achieved_updates_per_s": round(updates, 1),
                                "peak_updates_per_s": round(counter_peak, 1),
                                "frac": round(updates / counter_peak, 4),
                                "peak_source": "measured in this run (iso_probe_counter_rate)"},
                "updates_per_s": round(updates, 1),
                "stage_ms": {"surfaces": round(stage[0], 3), "distance_fields": round(stage[1], 3),
                             "histograms_nmi": round(stage[2], 3)}}
    # the other stages against their own algorithmic work: surfaces 4 V bytes
    # read (one pass over the volume for all isovalues) + 12 bytes per point
    # written, against HBM; distance fields as queries/s and (sample, point)
    # pairs/s (an exact search, latency-bound: not roofline-graded)
    surf_bytes = 4.0 * F + 12.0 * P
    roofline["stages"] = {
        "surfaces": {"algorithmic_bytes": surf_bytes, "achieved_gbs": round(surf_bytes / (stage[0] / 1e3) / 1e9, 2),
                     "frac_of_hbm": round(surf_bytes / (stage[0] / 1e3) / 1e9 / peak, 5), "points": P},
        "distance_fields": {"queries_per_s": round(m * F / (stage[1] / 1e3), 1),
                            "sample_point_pairs_per_s": round(float(F) * P / (stage[1] / 1e3), 1)},
    }

    line = {
        "metric": METRIC if args.config == 3 else "ISM pairs/sec",
        "value": round(value, 2),
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (reference FP32 MI)" if args.mi == "ref32" else "f32 (FP64 NMI)",
        "data": "synthetic (seeded)",
        "config": bench_config(args, name, n, bins, world),
        "method": {"surface": "marching cubes (reference frame)", "distance": args.df,
                   "mi": ("REF32: the reference's FP32 MI per ordered pair, bit-identical to its own kernel"
                          if args.mi == "ref32" else "FP64"),
                   "nonempty_surfaces": int(m), "pairs": int(pairs)},
        "e2e": {"value": round(world * pairs / (e2e_ms / 1e3), 2), "unit": "pairs/s",
                "h2d_bytes_per_step": int(F * 4 + n * 4), "d2h_bytes_per_step": int(m * m * 4 + m * 4)},
        "gpu_launches": int(launches),
        "tuning": tuning,
        "roofline": roofline,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_mi_other:
        other = "fp64" if args.mi == "ref32" else "ref32"
        line["mi_" + other] = other_mi_leg(ctx, step, d_vol, ism_dev, flush, stream, m, pairs, args.steps, other)
    if rank == 0 and not args.no_plain:
        line["plain"] = plain_leg(ctx, vol, isos, sstats, stage, pairs, value, args.plain_surfaces)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(vol, isos, bins, sample_scale=args.cpu_scale)
    if rank == 0 and args.serving_requests > 0:
        ctx.close()
        ctx = None
        batched, one, desc = serving_stats(args.serving_requests, args.rate, args.slots, args.budget_gb,
                                           mi=args.mi)
        line["serving"] = {"workload": desc, "continuous_batching": batched, "one_at_a_time": one}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ctx is not None:
        ctx.close()
    if pg is not None:
        pg.destroy_process_group()


TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "histogram_traffic__ism-256cubed-256iso-256bins.md")
HIST_SOURCE = os.path.join(PKG, "csrc", "iso_histogram.cu")


def histogram_traffic():
    """(DRAM bytes of the histogram stage per ISM, source) from the committed
    ncu summary, which records the sha256 of csrc/iso_histogram.cu it was
    captured on; (None, reason) when it is absent or that source changed."""
    import hashlib
    if not os.path.exists(TRAFFIC_PROFILE):
        return None, "no ncu summary committed for this workload"
    vals = {}
    with open(TRAFFIC_PROFILE) as f:
        for line in f:
            if ":" in line and line.strip().startswith("- `"):
                k, v = line.strip()[3:].split("`", 1)
                vals[k] = v.split(":", 1)[1].strip().strip("`")
    with open(HIST_SOURCE, "rb") as f:
        sha = hashlib.sha256(f.read()).hexdigest()
    if vals.get("source_sha256") != sha:
        return None, "ncu summary was captured on another histogram source"
    return float(vals["traffic_bytes_per_ism"]), "ncu capture (%s)" % os.path.relpath(TRAFFIC_PROFILE, ROOT)


def other_mi_leg(ctx, step, d_vol, ism_dev, flush, stream, m, pairs, steps, other):
    """The same ISM with the other MI evaluation ("fp64": the engine's FP64
    NMI; "ref32": the reference's own FP32 evaluation per ordered pair, bit for
    bit its kernel's map), timed like the headline (device-resident, L2
    flushed, CUDA events), and the largest difference between the two maps."""
    import torch

    import isosim
    main_map = ism_dev[:m * m].cpu().numpy().reshape(m, m).copy()
    main_mode = isosim.MI_REF32 if other == "fp64" else isosim.MI_FP64
    ctx.set_mi_mode(isosim.MI_FP64 if other == "fp64" else isosim.MI_REF32)
    try:
        step(d_vol, ism_dev)
        ms = 0.0
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            _, _, _, timing = step(d_vol, ism_dev)
            ev1.record(stream)
            ev1.synchronize()
            ms += ev0.elapsed_time(ev1)
        ms /= steps
        other_map = ism_dev[:m * m].cpu().numpy().reshape(m, m)
    finally:
        ctx.set_mi_mode(main_mode)
    return {"value": round(pairs / (ms / 1e3), 2), "unit": "pairs/s", "ms_per_ism": round(ms, 3),
            "histograms_nmi_ms": round(timing.histogram_ms, 3),
            "max_abs_diff_vs_headline_map": float(np.abs(other_map - main_map).max()),
            "note": ("the engine's FP64 NMI (accurate; differs from the reference's FP32 map by the reference's "
                     "own rounding)" if other == "fp64" else
                     "the reference's FP32 MI evaluation per ordered pair, bit-identical to its own kernel")}


def plain_leg(ctx, vol, isos, sstats, stage, pairs, value, k_surfaces):
    """The plain single-launch FP32 GPU path: the same surfaces and histograms,
    with each distance field computed by brute force on the CUDA cores
    (df_brute_kernel: every sample against every surface point).  The brute
    force over all n surfaces takes minutes at 256^3, so it runs on
    k_surfaces sampled surfaces and is scaled to the whole ISM by
    (sample, point) pairs -- its work is exactly F*P per surface.  The same
    surfaces also go through the tensor-core brute force (ISO_DF_TC: the
    contraction on tcgen05 plus exact FP32 candidates), reported beside it."""
    import isosim
    dims = vol.shape
    F = int(np.prod(dims))
    n = len(isos)
    counts = np.array([sstats[k].points for k in range(n)], np.int64)
    nonempty = np.nonzero(counts)[0]
    pick = nonempty[np.linspace(len(nonempty) // 4, 3 * len(nonempty) // 4, k_surfaces).astype(int)]
    pts, _ = ctx.surface_points(vol.ravel(), dims, isos[pick], surface=isosim.SURFACE_MC, frame=isosim.FRAME_REF)
    out = {}
    for key, method in (("brute_fp32", isosim.DF_BRUTE), ("tensor_core", isosim.DF_TC)):
        work, secs = 0.0, 0.0
        for p in pts:
            pn = (p / np.float32(max(dims))).astype(np.float32)
            ctx.distance_field(pn[:300], dims, method=method)  # warm-up
            t0 = time.perf_counter()
            ctx.distance_field(pn, dims, method=method)
            secs += time.perf_counter() - t0
            work += float(F) * len(p)
        rate = work / secs
        df_s = float(F) * float(counts.sum()) / rate
        t_ism = (stage[0] + stage[2]) / 1e3 + df_s
        out[key] = {"value": round(pairs / t_ism, 2), "unit": "pairs/s", "seconds_per_ism": round(t_ism, 2),
                    "sample_point_pairs_per_s": float("%.4g" % rate)}
    plain = out["brute_fp32"]["value"]
    return {"value": plain, "unit": "pairs/s", "extrapolated": True,
            "distance": "brute-force FP32 (df_brute_kernel)", "seconds_per_ism": out["brute_fp32"]["seconds_per_ism"],
            "sample": "%d of %d surfaces (%d points) timed by brute force on the CUDA cores and on the tensor cores, "
                      "scaled to all %d surface points by (sample, point) pairs; surfaces and histograms as measured "
                      "above" % (len(pts), len(nonempty), int(sum(len(p) for p in pts)), int(counts.sum())),
            "brute_sample_point_pairs_per_s": out["brute_fp32"]["sample_point_pairs_per_s"],
            "tensor_core": out["tensor_core"],
            "batched_over_plain": round(value / plain, 1)}


def cpu_baseline(vol, isos, bins, sample_scale=1.0):
    """The pipeline's CPU arithmetic on all host cores over a bounded sample,
    scaled to one full ISM (extrapolated):
      marching cubes of a few isovalues (the oracle's restatement of the
      reference kernels), distance fields of a random sample of voxels through
      a k-d tree (exact, same canonical distance), joint histograms + FP32 NMI
      of a few field pairs (the oracle's restatement, bit-exact with the
      reference's calculate_histogram_CPU)."""
    from concurrent.futures import ThreadPoolExecutor

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    dims = vol.shape
    X, Y, Z = dims
    F = X * Y * Z
    n = len(isos)
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(0)
    k_iso = max(2, int(4 * sample_scale))
    iso_idx = np.linspace(n // 8, n - 1 - n // 8, k_iso).astype(int)

    def mc(i):
        t0 = time.perf_counter()
        pts = oracle.marching_cubes(vol, dims, float(isos[i]), frame=0)[0]
        return pts, time.perf_counter() - t0

    with ThreadPoolExecutor(min(cores, k_iso)) as ex:
        res = list(ex.map(mc, iso_idx))
    t_mc = float(np.mean([t for _, t in res]))
    n_samp = max(1024, int(4096 * sample_scale))

    def df(pts):
        # tree build + a random sample of queries, each timed inside the C code
        p = oracle.normalize_points(pts, dims)
        idx = np.random.default_rng(len(pts)).integers(0, F, n_samp)
        _, t_build, t_query = oracle.distance_field_kd_timed(p, dims, idx)
        return t_build + t_query / n_samp * F

    surfaces = [p for p, _ in res if len(p)]
    with ThreadPoolExecutor(min(cores, len(surfaces))) as ex:
        t_df = float(np.mean(list(ex.map(df, surfaces))))
    k_pairs = max(cores, int(cores * sample_scale))
    f = np.abs(rng.standard_normal((2, F))).astype(np.float32) * 0.3
    lo = [oracle.field_interval(x) for x in f]

    def pair(_):
        t0 = time.perf_counter()
        joint, cs, rs = oracle.pair_histogram(f[0], f[1], bins, lo[0], lo[1])
        oracle.mi_f32(joint, cs, rs, F)
        return time.perf_counter() - t0

    with ThreadPoolExecutor(cores) as ex:
        t_pair = float(np.mean(list(ex.map(pair, range(k_pairs)))))
    pairs = n * (n - 1) // 2
    t_ism = (n * (t_mc + t_df) + pairs * t_pair) / cores
    return {"value": round(pairs / t_ism, 4), "unit": "pairs/s", "cores": cores, "kind": "port",
            "sample": "%d isovalues of marching cubes, %d k-d-tree distance samples per surface, %d histogram "
                      "pairs; per-unit single-core times scaled to one %d-isovalue ISM on %d cores (extrapolated)"
                      % (k_iso, n_samp, k_pairs, n, cores),
            "seconds_per_ism": round(t_ism, 2),
            "per_unit_s": {"marching_cubes_per_isovalue": round(t_mc, 4), "distance_field_per_isovalue": round(t_df, 4),
                           "histogram_nmi_per_pair": round(t_pair, 5)}}


REF_HIST_FIELDS = 88        # 88^2 ordered pairs x 256^2 bins x 4 B = 2.03 GB: one run under the 2 GiB cap
REF_HIST_VALUES = 999999    # one 1,000,000-value chunk (JointHistogram.cu:21), its last-chunk path


def reference_gpu(vol, isos, bins, k_surfaces=4):
    """The reference's own kernels on this GPU (its sources compiled into
    oracle/_ref cubins, driven by oracle/refgpu.py with its host steps), as
    device time measured with CUDA events around each launch, on a bounded
    sample scaled to one ISM:
      * marching cubes of k_surfaces isovalues: classifyVoxel, compactVoxels,
        generateTriangles (MarchingCube.cu; its thrust scans, vertex sort and
        host copies not counted);
      * the LBVH distance field of each of those surfaces over every voxel:
        Morton, build, box and traversal kernels (BVH.cu; its thrust sort not
        counted);
      * one histogram run of calculate_histogram_g: REF_HIST_FIELDS fields of
        REF_HIST_VALUES values, i.e. 7,744 ordered pairs in one launch (a
        full run: the reference packs 8,192 pairs of 256 bins into its 2 GiB
        allocation), scaled to the n^2 ordered pairs and F values of the
        workload's map.
    Only what the reference's kernels spend on the GPU counts, so the figure
    is an upper bound on its throughput.  None when a cubin or the GPU is
    missing."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import oracle
        import refgpu
        if not (refgpu.available() and refgpu.mc_available() and refgpu.bvh_available()):
            return None
        refgpu._driver()
    except Exception as e:  # no GPU or no driver
        return {"unavailable": "reference kernels not run: %s" % str(e).splitlines()[0][:160]}
    dims = vol.shape
    F = int(np.prod(dims))
    n = len(isos)
    flat = np.ascontiguousarray(vol, np.float32).ravel()
    pick = np.linspace(n // 4, 3 * n // 4, k_surfaces).astype(int)
    t_mc, t_bvh, skipped, points = {}, {}, [], []
    for k in pick:
        pts, _, _ = refgpu.marching_cubes(flat, dims, float(isos[k]), timing=t_mc)
        if len(pts) < 2:
            skipped.append(int(k))
            continue
        try:
            refgpu.lbvh_distance_field(oracle.normalize_points(pts, dims), dims, timing=t_bvh)
            points.append(len(pts))
        except ValueError:
            skipped.append(int(k))   # a tree the check refuses: not run
    done = len(points)
    if done == 0:
        return {"unavailable": "no sampled surface passed the reference tree check"}
    rng = np.random.default_rng(7)
    base = rng.uniform(0.0, 1.0, REF_HIST_VALUES)
    fields = np.stack([np.abs(base * (1 + 0.02 * q) + 0.1 * rng.standard_normal(REF_HIST_VALUES))
                       for q in range(REF_HIST_FIELDS)]).astype(np.float32)
    t_hist = {}
    refgpu.similarity(fields, bins, timing=t_hist)
    ms_mc = sum(t_mc.values()) / len(pick)
    ms_bvh = sum(t_bvh.values()) / done
    ms_hist = t_hist["calculate_histogram_g"] * (n * n) / REF_HIST_FIELDS ** 2 * F / REF_HIST_VALUES
    s_ism = (n * (ms_mc + ms_bvh) + ms_hist) / 1e3
    pairs = n * (n - 1) // 2
    return {"value": round(pairs / s_ism, 4), "unit": "pairs/s", "kind": "reference kernels, device time",
            "seconds_per_ism": round(s_ism, 2),
            "per_unit_ms": {"marching_cubes_per_isovalue": round(ms_mc, 3),
                            "lbvh_per_surface": round(ms_bvh, 3),
                            "histogram_run_launch": round(t_hist["calculate_histogram_g"], 3),
                            "histograms_per_ism": round(ms_hist, 1)},
            "kernels_ms": {k: round(v, 3) for d in (t_mc, t_bvh, t_hist) for k, v in d.items()},
            "sample": "%d isovalues (%s) of marching cubes and LBVH fields over all %d voxels%s; one histogram "
                      "launch of %d fields x %d values (%d ordered pairs) scaled to %d ordered pairs x %d values "
                      "(extrapolated)" % (done, ",".join(str(int(k)) for k in pick if int(k) not in skipped), F,
                                          "; skipped %s" % skipped if skipped else "", REF_HIST_FIELDS,
                                          REF_HIST_VALUES, REF_HIST_FIELDS ** 2, n * n, F)}


def run_reference(args):
    """The reference arm: the pipeline's arithmetic on the host cores (the
    CPU restatements under oracle/: the reference's own compiled parts do not
    build on the GPU host), never the engine.  Each step is one bounded
    sample of the workload (cpu_baseline); ms_per_step is that sample's real
    duration and value the sample's per-unit rates scaled to whole ISMs."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    vol, isos, bins, name = workload(args.config)
    n = len(isos)
    for _ in range(args.warmup):
        cpu_baseline(vol, isos, bins, sample_scale=args.ref_scale)
    vals, secs = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        vals.append(cpu_baseline(vol, isos, bins, sample_scale=args.ref_scale))
        secs.append(time.perf_counter() - t0)
    v = float(np.median([c["value"] for c in vals]))
    ref_gpu = None if args.no_ref_gpu else reference_gpu(vol, isos, bins)
    cb = dict(vals[0])
    cb["value"] = round(v, 4)
    line = {"metric": METRIC if args.config == 3 else "ISM pairs/sec", "value": round(v, 4), "unit": "pairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * float(np.mean(secs)), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "impl": "reference", "extrapolated": True,
            "step": "one bounded sample per step: " + cb["sample"],
            "config": bench_config(args, name, n, bins, world),
            "cpu_baseline": cb,
            "e2e": {"value": round(v, 4), "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if ref_gpu is not None:
        line["reference_gpu"] = ref_gpu
    print(json.dumps(line), flush=True)


def serving_stats(requests, rate, slots, budget_gb, max_wait_ms=2000.0, mi="ref32"):
    """Poisson stream of ISM requests through the serving loop (continuous
    batching under an HBM budget) and through one-request-at-a-time serving.
    Shapes, isovalue counts and bins are drawn per request (seeded); volumes
    come from a small pool of seeded blob and k^-3 fields kept on the device.
    Returns (batched, one_at_a_time, workload description)."""
    import torch

    import isosim
    import isosim.synth as synth

    rng = np.random.default_rng(5000)
    shapes = [(64, 64, 64), (128, 128, 128), (192, 128, 128), (256, 256, 256), (600, 248, 248)]
    pool = {}
    for k, sh in enumerate(shapes):
        scale = min(sh) / 64.0
        pool[(sh, "blobs")] = torch.from_numpy(
            synth.gaussian_blobs(sh, 8, 5100 + k, sigma=(4.0 * scale, 12.0 * scale)).ravel()).cuda()
        if np.prod(sh) <= 192 * 128 * 128:
            pool[(sh, "grf")] = torch.from_numpy(synth.power_law_field(sh, 3.0, 5200 + k).ravel()).cuda()
    reqs = []
    t = 0.0
    for r in range(requests):
        t += rng.exponential(1.0 / rate)
        sh = shapes[rng.integers(len(shapes))]
        kind = "grf" if (sh, "grf") in pool and rng.random() < 0.5 else "blobs"
        n = int(rng.choice([16, 32, 64, 128, 256]))
        bins = int(rng.choice([128, 256]))
        vol = pool[(sh, kind)]
        if kind == "grf":
            isos = np.linspace(-2.5, 2.5, n).astype(np.float32)
        else:
            lo, hi = float(vol.min()), float(vol.max())
            isos = np.array([lo + (i + 1) * (hi - lo) / (n + 1) for i in range(n)], np.float32)
        reqs.append((t, vol, sh, isos, bins))

    costs = np.array([float(np.prod(sh)) * len(isos) * (len(isos) + 64) for (_, _, sh, isos, _) in reqs])
    small = costs <= np.median(costs)

    def serve(slots, policy):
        with isosim.Server(0, slots=slots, budget_bytes=int(budget_gb * (1 << 30))) as srv:
            srv.set_policy(policy, max_wait_ms)
            srv.set_mi_mode(isosim.MI_REF32 if mi == "ref32" else isosim.MI_FP64)
            # warm each worker's arena on a small request
            for _ in range(slots):
                srv.wait(srv.submit(pool[(shapes[0], "blobs")], shapes[0], reqs[0][3][:16], bins=128))
            t0 = time.perf_counter()
            tickets = []
            for (at, vol, sh, isos, bins) in reqs:
                delay = t0 + at - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets.append((srv.submit(vol, sh, isos, bins=bins), time.perf_counter()))
            pairs, lat, lat_small, failed = 0, [], [], 0
            for q, (tk, _) in enumerate(tickets):
                try:
                    ism, ids, res = srv.wait(tk)
                except isosim.IsoError:
                    failed += 1
                    continue
                pairs += len(ids) * (len(ids) - 1) // 2
                lat.append(res.latency_ms)
                if small[q]:
                    lat_small.append(res.latency_ms)
            wall = time.perf_counter() - t0
            st = srv.stats()
        lat = np.array(lat)
        return {"pairs_per_s": round(pairs / wall, 1), "wall_s": round(wall, 2), "pairs": int(pairs), "failed": failed,
                "p50_ms": round(float(np.percentile(lat, 50)), 1), "p99_ms": round(float(np.percentile(lat, 99)), 1),
                "small_request_p50_ms": round(float(np.percentile(lat_small, 50)), 1) if lat_small else None,
                "policy": "shortest first" if policy == isosim.SERVE_SHORTEST_FIRST else "fifo",
                "peak_admitted_gb": round(st.peak_device_bytes / (1 << 30), 2)}

    batched = serve(slots, isosim.SERVE_SHORTEST_FIRST)
    plain = serve(1, isosim.SERVE_FIFO)
    desc = ("Poisson stream of %d requests at %g req/s; shapes %s; isovalues {16..256}; bins {128,256}; "
            "%g GB HBM budget; %d slots; %s MI; small requests: work estimate at or below the median"
            % (requests, rate, shapes, budget_gb, slots,
               "the reference's FP32" if mi == "ref32" else "FP64"))
    return batched, plain, desc


def run_serving(args):
    batched, plain, desc = serving_stats(args.requests, args.rate, args.slots, args.budget_gb, mi=args.mi)
    line = {"metric": "ISM pairs/sec and p50/p99 latency, serving", "value": batched["pairs_per_s"],
            "unit": "pairs/s", "n_gpus": 1, "higher_is_better": True, "data": "synthetic (seeded)",
            "config": {"workload": desc, "slots": args.slots},
            "continuous_batching": batched, "one_at_a_time": plain}
    print(json.dumps(line), flush=True)


class _OneRank:
    """torch.distributed stand-in for a single process."""

    @staticmethod
    def all_gather(out, t):
        out[0].copy_(t)

    @staticmethod
    def gather(t, outs, dst=0):
        outs[0].copy_(t)

    @staticmethod
    def barrier():
        pass


def run_multi(args):
    """Multi-volume batch: V variables x T timesteps of S^3 k^-3 fields advected
    0.5 voxel/step and mixed per variable (seeded 4x4 blend + tanh); 64
    isovalues per volume -> one ISM each, 16 representatives each, then all
    16x16 cross maps (same variable across timesteps, all variables at equal
    timesteps), aggregated into TSM/VSM entries.  Under torchrun the volumes
    are sharded over ranks; one all-gather of representative fields, then each
    rank computes its share of the cross-map blocks in one launch."""
    import torch

    import isosim
    from isosim import multi

    world, rank, local, pg = dist_init()
    torch.cuda.set_device(local)
    dist = pg if pg is not None else _OneRank
    V, T, S, n, bins, reps = args.variables, args.timesteps, args.size, 64, 128, 16
    g = torch.Generator(device="cuda").manual_seed(4000)
    shape = (S, S, S)
    k = torch.fft.fftfreq(S, device="cuda")
    kr = torch.fft.rfftfreq(S, device="cuda")
    kk = torch.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + kr[None, None, :] ** 2)
    amp = kk.clamp_min(1e-12) ** -1.5
    amp[0, 0, 0] = 0
    bases = [torch.fft.rfftn(torch.randn(shape, generator=g, device="cuda")) * amp for _ in range(4)]
    vel = torch.randn(3, generator=g, device="cuda")
    vel = 0.5 * vel / vel.norm()
    blend = torch.randn(4, 4, generator=g, device="cuda")

    def volume(var, t):
        phase = torch.exp(-2j * np.pi * t * (vel[0] * k[:, None, None] + vel[1] * k[None, :, None] +
                                             vel[2] * kr[None, None, :]))
        fields = [torch.fft.irfftn(b * phase, s=shape) for b in bases]
        fields = [(f - f.mean()) / f.std() for f in fields]
        mix = sum(blend[var, j] * fields[j] for j in range(4))
        return torch.tanh(mix / mix.std()).contiguous().ravel()

    F = S ** 3
    stride = (F + 63) // 64 * 64
    ctx = isosim.Context(local)
    stats = {"ism_pairs": 0, "t_ism": 0.0, "stage_ms": np.zeros(3), "t_parts": np.zeros(3)}

    # this rank's volumes are generated before the timed batch (the engine's
    # input, like a volume loaded from disk)
    vlo, vhi = multi.shard(V * T, rank, world)
    volumes = {vid: volume(vid // T, vid % T) for vid in range(vlo, vhi)}
    torch.cuda.synchronize()

    def local_fields(lo, hi):
        rows = torch.zeros(((hi - lo) * reps, stride), dtype=torch.float32, device="cuda")
        for vid in range(lo, hi):
            vol = volumes[vid]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            vmin, vmax = ctx.real_range(vol)  # the engine's device reduction
            isos = np.array([vmin + (i + 1) * (vmax - vmin) / (n + 1) for i in range(n)], np.float32)
            t1 = time.perf_counter()
            ism, ids, _, timing = ctx.ism(vol, shape, isos, bins=bins)
            t2 = time.perf_counter()
            stats["ism_pairs"] += len(ids) * (len(ids) - 1) // 2
            stats["stage_ms"] += [timing.surface_ms, timing.distance_ms, timing.histogram_ms]
            picks = sorted(r[3] for r in isosim.select_representatives(ism, ids, isos, reps))
            for q, row in enumerate(picks):
                ctx.copy_field(row, rows[(vid - lo) * reps + q])
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            stats["t_ism"] += t3 - t0
            stats["t_parts"] += [t1 - t0, t2 - t1, t3 - t2]
        return rows

    R = V * T * reps
    pmap = torch.zeros((R, R), dtype=torch.float32, device="cuda")

    def pair_values(fields, pairs):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.pair_map(fields, pairs, bins=bins, n=F, stride=stride, out=pmap)
        out = pmap.cpu().numpy()[pairs[:, 0], pairs[:, 1]]
        stats["t_cross"] = time.perf_counter() - t0
        stats["cross_pairs"] = len(pairs)
        return out

    barrier(pg)
    t0 = time.perf_counter()
    full, blocks = multi.run_batch(dist, rank, world, V, T, reps, local_fields, pair_values)
    torch.cuda.synchronize()
    barrier(pg)
    wall = max_over_ranks(pg, time.perf_counter() - t0)
    ism_pairs = stats["ism_pairs"]
    if pg is not None:
        tot = torch.tensor([float(ism_pairs)], dtype=torch.float64, device="cuda")
        pg.all_reduce(tot)
        ism_pairs = int(tot.item())
    if rank == 0:
        agg = ctx.block_similarity(full, reps, blocks)
        cross = len(blocks) * reps * reps
        isms = V * T
        line = {"metric": "ISM + cross-map pairs/sec, multi-volume batch",
                "value": round((ism_pairs + cross) / wall, 1),
                "unit": "pairs/s", "n_gpus": world, "higher_is_better": True, "scaling": "strong",
                "data": "synthetic (seeded, generated on the GPU)",
                "config": {"workload": "%d variables x %d timesteps of %d^3, %d isovalues, %d representatives, %d bins"
                                       % (V, T, S, n, reps, bins), "isms": isms, "cross_maps": len(blocks),
                           "parallelism": "volumes sharded over %d rank(s); one all-gather of representative "
                                          "fields" % world},
                "wall_s": round(wall, 3),
                "rank0_ism_stage": {"pairs": int(stats["ism_pairs"]), "seconds": round(stats["t_ism"], 3),
                                    "engine_stage_s": {k: round(float(v) / 1e3, 3) for k, v in
                                                       zip(("surfaces", "distance_fields", "histograms_nmi"),
                                                           stats["stage_ms"])},
                                    "host_s": {k: round(float(v), 3) for k, v in
                                               zip(("isovalue_range", "ism_call", "representatives_and_copies"),
                                                   stats["t_parts"])}},
                "rank0_cross_stage": {"pairs": int(stats.get("cross_pairs", 0)),
                                      "seconds": round(stats.get("t_cross", 0.0), 3)},
                "tsm_vsm_sample": {"first_blocks": [[int(a), int(b), round(float(x), 4), round(float(y), 4)]
                                                    for (a, b), (x, y) in zip(blocks[:4], agg[:4])]}}
        print(json.dumps(line), flush=True)
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()


def run_case(case, hist_seg=None, hist_codes=None):
    """Small fixed workloads for kernel profiles: 'hist-small' = similarity
    map of 16 distance-like fields of 128^3 values at 256 bins; 'pipe-small' =
    the 64^3, 32-isovalue, 128-bin pipeline; 'ism-128' = the 128^3 blob+noise
    volume with 64 isovalues and 256 bins (distance fields of real surfaces)."""
    import isosim
    import isosim.synth as synth
    ctx = isosim.Context(0)
    if hist_seg is not None:
        ctx.set_hist_segment_values(hist_seg)
    if hist_codes is not None:
        ctx.set_hist_row_codes(hist_codes)
    if case == "seg-small":
        # 160^3 blob + noise volume, 32 isovalues, 256 bins: fields of 4,096,000
        # values, two segments each (the segment-major kernels)
        vol, isos, bins = synth.config3(size=160, n=32)
        for _ in range(2):
            ctx.ism(vol.ravel(), (160, 160, 160), isos, bins=bins)
    elif case == "ism-ref32":
        # the 256^3 benchmark ISM with the reference's own FP32 MI (every
        # ordered pair's joint histogram kept, then mi_ref32_kernel)
        vol, isos, bins = synth.config3()
        ctx.set_mi_mode(isosim.MI_REF32)
        for _ in range(2):
            ctx.ism(vol.ravel(), (256, 256, 256), isos, bins=bins)
    elif case == "tc-small":
        # one surface of the 128^3 k^-3 field through the tensor-core distance
        # kernel (and the LBVH for comparison)
        vol, isos, _ = synth.config2()
        pts, _ = ctx.surface_points(vol.ravel(), (128, 128, 128), isos[[50]])
        pn = (pts[0] / np.float32(128)).astype(np.float32)
        for _ in range(2):
            ctx.distance_field(pn, (128, 128, 128), method=isosim.DF_TC)
    elif case == "ism-128":
        vol, isos, bins = synth.config3(size=128, n=64)
        for _ in range(2):
            ctx.ism(vol.ravel(), (128, 128, 128), isos, bins=bins)
    elif case == "hist-small":
        rng = np.random.default_rng(0)
        n = 128 ** 3
        base = rng.uniform(0, 1, n)
        f = np.stack([np.abs(base * (1 + 0.25 * k) + 0.15 * rng.standard_normal(n)) for k in range(16)]).astype(np.float32)
        for _ in range(2):
            ctx.similarity_map(f, 256)
    else:
        vol, isos, bins = synth.config1()
        for _ in range(2):
            ctx.ism(vol.ravel(), (64, 64, 64), isos, bins=bins)
    ctx.close()
    print("case", case, "ok")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=3, choices=[1, 2, 3])
    ap.add_argument("--df", default="lbvh", choices=["lbvh", "brute", "tc"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--hist-seg", type=int, default=None,
                    help="segment length of the segment-major histogram schedule (0: fused kernel only)")
    ap.add_argument("--hist-traffic", type=float, default=None,
                    help="DRAM bytes per histogram launch from an ncu capture (reported as roofline.traffic)")
    ap.add_argument("--cpu-scale", type=float, default=1.0)
    ap.add_argument("--ref-scale", type=float, default=0.5,
                    help="sample size of each reference-arm step (see cpu_baseline)")
    ap.add_argument("--no-plain", action="store_true", help="skip the brute-force plain-path leg")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no autotuner)")
    ap.add_argument("--mi", default="ref32", choices=["ref32", "fp64"],
                    help="MI evaluation of the timed ISM: the reference's own FP32 evaluation (ISO_MI_REF32, "
                         "bit-identical to its kernel) or the engine's FP64 NMI")
    ap.add_argument("--no-mi-other", action="store_true",
                    help="skip the timing of the other MI evaluation")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="reference arm: skip the timing of the reference's own kernels on the GPU")
    ap.add_argument("--hist-codes", type=int, default=None, choices=[0, 1],
                    help="segment-major histograms with (1) or without (0) precomputed row buckets")
    ap.add_argument("--plain-surfaces", type=int, default=2)
    ap.add_argument("--serving-requests", type=int, default=24,
                    help="requests of the serving leg in the default line (0: none)")
    ap.add_argument("--case", default=None, choices=["hist-small", "pipe-small", "ism-128", "tc-small", "seg-small", "ism-ref32"],
                    help="run a small fixed case twice and exit (profiling target)")
    ap.add_argument("--mode", default="single", choices=["single", "serving", "multi"])
    ap.add_argument("--requests", type=int, default=40)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--variables", type=int, default=4)
    ap.add_argument("--timesteps", type=int, default=50)
    ap.add_argument("--size", type=int, default=128)
    args = ap.parse_args()
    if args.case:
        run_case(args.case, args.hist_seg, args.hist_codes)
    elif args.mode == "serving":
        run_serving(args)
    elif args.mode == "multi":
        run_multi(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
