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
restatement of its surface and distance stages on the host cores.
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


def workload(config):
    import isosim.synth as synth
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
    method = isosim.DF_LBVH if args.df == "lbvh" else isosim.DF_BRUTE
    ctx = isosim.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    d_vol = torch.from_numpy(vol.ravel()).to(f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    n = len(isos)
    ism_dev = torch.empty(n * n, dtype=torch.float32, device=f"cuda:{local}")

    def step(vol_arg, out):
        return ctx.ism(vol_arg, (X, Y, Z), isos, surface=isosim.SURFACE_MC, frame=isosim.FRAME_REF,
                       df_method=method, bins=bins, out=out)

    for _ in range(args.warmup):
        _, ids, _, timing = step(d_vol, ism_dev)
    m = len(ids)
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
    hist_s = stage[2] / 1e3
    peak, peak_kind = load_peaks()
    achieved = hist_bytes / hist_s / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": None,
                "kernel": "joint_histogram_mi_kernel",
                "peak_source": peak_kind,
                "updates_per_s": round(F * pairs / hist_s, 1),
                "stage_ms": {"surfaces": round(stage[0], 3), "distance_fields": round(stage[1], 3),
                             "histograms_nmi": round(stage[2], 3)}}

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
        "dtype": "f32 (FP64 NMI)",
        "data": "synthetic (seeded)",
        "config": {"workload": name, "isovalues": int(n), "nonempty_surfaces": int(m), "pairs": int(pairs),
                   "bins": int(bins), "surface": "marching cubes (reference frame)",
                   "distance": args.df, "l2": "256 MB flush before every timed step",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": round(world * pairs / (e2e_ms / 1e3), 2), "unit": "pairs/s",
                "h2d_bytes_per_step": int(F * 4 + n * 4), "d2h_bytes_per_step": int(m * m * 4 + m * 4)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(vol, isos, bins, sample_scale=args.cpu_scale)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()


def cpu_baseline(vol, isos, bins, sample_scale=1.0):
    """Reference arithmetic on the host cores over a bounded sample, scaled to
    one full ISM: marching cubes of a few isovalues, FP32 distance fields of a
    sample of voxels, joint histograms + NMI of a sample of pairs (the oracle's
    FP32 histogram/NMI restatement is bit-exact with the reference's
    calculate_histogram_CPU)."""
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
    iso_idx = np.linspace(0, n - 1, k_iso).astype(int)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        surfs = list(ex.map(lambda i: oracle.marching_cubes(vol, dims, float(isos[i]), frame=0)[0], iso_idx))
    t_mc = (time.perf_counter() - t0) / k_iso * min(cores, k_iso)  # per isovalue, one core
    # distance fields: a random subset of sample points of each surface
    n_samp = max(256, int(1024 * sample_scale))
    pts_all = [oracle.normalize_points(p, dims) for p in surfs if len(p)]
    t0 = time.perf_counter()
    evals = 0
    for p in pts_all:
        # emulate the per-voxel scan: distance of n_samp random grid points to all points
        sub = rng.integers(0, F, n_samp)
        s = np.stack([(sub // (Y * Z)) / np.float32(X), ((sub // Z) % Y) / np.float32(Y), (sub % Z) / np.float32(Z)], 1)
        s = s.astype(np.float32)
        for q in range(0, n_samp, 64):
            d = ((s[q:q + 64, None, :] - p[None, :, :]) ** 2).sum(-1).min(1)
        evals += n_samp * len(p)
    t_df_eval = (time.perf_counter() - t0) / max(evals, 1)
    mean_p = np.mean([len(p) for p in pts_all]) if pts_all else 0
    # histograms: fields from the sampled surfaces' exact DF would be too slow;
    # use fields of the right size and distribution (the cost is value-independent)
    k_pairs = max(cores, int(2 * cores * sample_scale))
    f = np.abs(rng.standard_normal((2, F))).astype(np.float32)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda _: oracle.pair_histogram(f[0], f[1], bins), range(k_pairs)))
    wall = time.perf_counter() - t0
    t_pair = wall / k_pairs  # wall per pair with `cores` threads
    pairs = n * (n - 1) // 2
    t_ism = (n * t_mc / cores) + (F * mean_p * n * t_df_eval / cores) + pairs * t_pair
    return {"value": round(pairs / t_ism, 4), "unit": "pairs/s", "cores": cores, "kind": "port",
            "sample": "%d isovalues of marching cubes, %d sample voxels per distance field, %d histogram pairs, "
                      "scaled to one %d-isovalue ISM (extrapolated)" % (k_iso, n_samp, k_pairs, n),
            "seconds_per_ism": round(t_ism, 2)}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    vol, isos, bins, name = workload(args.config)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(vol, isos, bins, sample_scale=0.5)
    for _ in range(args.steps):
        vals.append(cpu_baseline(vol, isos, bins, sample_scale=0.5))
    v = float(np.median([c["value"] for c in vals]))
    cb = dict(vals[0])
    cb["value"] = round(v, 4)
    line = {"metric": METRIC if args.config == 3 else "ISM pairs/sec", "value": round(v, 4), "unit": "pairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * (len(isos) * (len(isos) - 1) // 2) / v, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": name, "note": "host cores; reference arithmetic; extrapolated from a sample"},
            "cpu_baseline": cb,
            "e2e": {"value": round(v, 4), "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_case(case):
    """Small fixed workloads for kernel profiles: 'hist-small' = similarity
    map of 16 distance-like fields of 128^3 values at 256 bins; 'pipe-small' =
    the 64^3, 32-isovalue, 128-bin pipeline."""
    import isosim
    import isosim.synth as synth
    ctx = isosim.Context(0)
    if case == "hist-small":
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
    ap.add_argument("--df", default="lbvh", choices=["lbvh", "brute"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-scale", type=float, default=1.0)
    ap.add_argument("--case", default=None, choices=["hist-small", "pipe-small"],
                    help="run a small fixed case twice and exit (profiling target)")
    args = ap.parse_args()
    if args.case:
        run_case(args.case)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
