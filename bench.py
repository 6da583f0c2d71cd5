"""Benchmark of the CVT hot path (plain Lloyd, the reference's gCVT loop).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: 4096 x 4096 float32 density (1 + 32 seeded Gaussians, 0 outside the
disk of radius 0.48), 262,144 seeded sites uniform in the disk, no fixed
sites.  One step = the gCVT computation on it: load the inputs, 100 Lloyd
iterations with the reference's omega schedule (no early stop), the final
labelling pass.  Every step is a full Lloyd run from the same initial sites;
the density (64 MB) and site grid (64 MB) exceed no cache individually but the
loop's working set fits in L2 between iterations, so the L2 is flushed before
each step (config.l2).

Metric: Gpix-pass/s = n^2 x labelling passes / second, 101 passes per step
(100 Lloyd iterations + the final labelling), whole job over all GPUs.
  value : inputs resident in HBM (device-to-device load), CUDA events on the
          launching stream, max over ranks.
  e2e   : the same through the C ABI with pinned host buffers: host->device
          copies of sites, density and mask and the device->host copy of the
          label grid inside every timed step.
  roofline: one Lloyd iteration, the launch pair k_list + k_cell<0> (89.5 % +
          3.9 % of the run's device time): algorithmic bytes per iteration /
          its mean duration over iterations 2-100 of the timed steps (CUDA
          events on the launching stream around them) against the measured
          HBM copy bandwidth.
--impl reference runs the reference's algorithm on the host cores (the
oracle's OpenMP restatement of gcvt.cu, all threads) on a bounded sample of
the same workload, in the same unit.
Multi-GPU: independent replicas, one per rank (weak scaling).
Other workloads, each with its own JSON line: --config plain_8192 (8192^2,
64 Gaussians, 1,048,576 sites, 100 iterations; the same contract),
--config batched_64 (64 charts of 256^2-2048^2 iterated together),
--config mesh_2048 (a mesh rasterised to 2048^2, then Lloyd, then the lift).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "surface-remesher_gb300")
for _p in (os.path.join(PKG, "python"), PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

CONFIG = "plain_4096"
PLAIN = ("plain_4096", "plain_8192", "plain_1024")  # the plain Lloyd workloads bench.py runs
SEED = 1
ITERS = 100
PASSES = ITERS + 1
METRIC = "Gpix-pass/s, plain Lloyd CVT (gCVT loop), 4096^2 grid, 262,144 sites, 100 iterations"


def metric_of(workload, n, nsites, iters=ITERS):
    if workload == CONFIG:
        return METRIC
    return "Gpix-pass/s, plain Lloyd CVT (gCVT loop), %d^2 grid, %s sites, %d iterations" % (
        n, format(nsites, ","), iters)
UNIT = "Gpix-pass/s"
# Algorithmic bytes of one Lloyd iteration (k_list + k_cell<0>): the density
# once over its row support (4 B per support pixel: every such pixel belongs
# to exactly one cell); the current site bitmap read by k_list and the bitmap
# two iterations ahead cleared by k_cell (1/8 B per pixel each); per site its
# list entry written and read (4 + 4 B), its word of the fixed-site bitmap
# read and its bit OR-ed into the next bitmap (8 + 8 B).
ALG_BYTES_PER_SUPPORT_PX = 4.0
ALG_BYTES_PER_PX = 0.125 + 0.125
ALG_BYTES_PER_SITE = 24.0
# dram__bytes_read.sum + dram__bytes_write.sum of k_list + k_cell<0> for one
# iteration of this workload (iteration 31 of a graph-replayed run, warm L2),
# from the ncu capture summarised in profiles/cell_kernel_plain_4096.md:
# k_list 789,248 + 264,448, k_cell 13,910,784 + 6,594,304 bytes.
NCU_TRAFFIC_BYTES = 21558784
# the same capture on the 8192^2 / 1,048,576-site workload (iteration 31,
# profiles/cell_kernel_plain_8192.md): k_list 13,138,176 + 3,403,520, k_cell
# 265,760,256 + 77,200,896 bytes
NCU_TRAFFIC = {"plain_4096": NCU_TRAFFIC_BYTES, "plain_8192": 359502848, "plain_1024": None}


def support_pixels(rho):
    """Pixels inside the per-row [first, last] span of nonzero density."""
    nz = rho != 0
    rows = nz.any(1)
    first = np.argmax(nz, 1)
    last = rho.shape[1] - 1 - np.argmax(nz[:, ::-1], 1)
    return int(((last - first + 1) * rows).sum())


def jfa_line(n, ms, stats, peak, halo=16):
    """Jump-flooding labelling of the workload's sites: logical passes n/2 ..
    1 plus 1; launches = one per step above halo/2 plus one fused tail (halo/2
    .. 1, 1), or one per pass for halo 0; algorithmic 8 B per pixel per launch
    (labels in and out)."""
    k, passes = 1, 1
    while 2 * k <= n // 2:
        k *= 2
    while k >= 1:
        passes += 1
        k //= 2
    tail = 1  # passes in the fused tail (halo 0: none, every pass its own launch)
    while halo and (1 << (tail - 1)) < halo:
        tail += 1
    launches = passes - tail + 1
    alg = 8.0 * n * n * launches
    return {"ms": ms, "logical_passes": passes, "launches": launches,
            "gpix_pass_per_s": n * n * passes / (ms / 1e3) / 1e9,
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / peak,
                         "algorithmic_bytes": alg},
            "mislabelled_px": stats[0], "farther_px": stats[1], "pixels": stats[2],
            "mislabel_rate": stats[0] / stats[2], "farther_rate": stats[1] / stats[2]}


JUMP_EVERY = 4  # learned runs: rounds of three plain iterations and one learned step


def time_to_energy_line(G, ctx, n, sites, rho, mask, conv_iters=1000, jump_every=JUMP_EVERY,
                        repeats=3):
    """Time until the energy is within 1e-4 of the energy after 1000 plain
    iterations (E_conv), for plain Lloyd, for Lloyd with the learned step
    (surface-remesher_gb300/data/step_mlp.npy) on one context, and for the same
    learned run through the batch API (persistent batched kernels, one MLP
    launch for the batch).  The device stops each run at the first iteration
    whose energy meets the target (gcvt_ctx_set_target_energy); CUDA events
    around the run on its stream; median of `repeats` after one warm-up."""
    from train_step_mlp import DATA, time_to_energy
    ctx.set_target_energy(0)
    ctx.load(sites, rho, mask)
    ctx.iterate(conv_iters)
    e_conv = ctx.info()["energy"]
    target = e_conv * (1 + 1e-4)

    def med(fn):
        fn()
        runs = [fn() for _ in range(repeats)]
        runs.sort(key=lambda r: r[0])
        return runs[len(runs) // 2]

    plain = med(lambda: time_to_energy(ctx, sites, rho, mask, target, False, 0, conv_iters))
    params = np.load(os.path.join(DATA, "step_mlp.npy"))
    lctx = G.Context(n)
    lctx.learning(True)
    lctx.set_mlp(params)
    learned = med(lambda: time_to_energy(lctx, sites, rho, mask, target, True, jump_every,
                                         conv_iters))
    batched = med(lambda: batched_time_to_energy(G, [lctx], [(sites, rho, mask)], [target],
                                                 params, jump_every, conv_iters))
    lctx.close()
    return {"target": "E <= (1 + 1e-4) E_conv, E_conv = energy after %d plain iterations"
                      % conv_iters,
            "e_conv": e_conv, "stop": "on the device at the first iteration meeting the target",
            "plain_ms": plain[0] * 1e3, "plain_iterations": plain[1],
            "learned_ms": learned[0] * 1e3, "learned_iterations": learned[1],
            "jumps_tried": learned[2], "jumps_kept": learned[3], "jump_every": jump_every,
            "learned_over_plain": plain[0] / learned[0],
            "learned_batched_ms": batched[0] * 1e3, "learned_batched_iterations": batched[1],
            "learned_batched_over_plain": plain[0] / batched[0]}


def batched_time_to_energy(G, ctxs, inputs, targets, params, jump_every, limit):
    """(seconds, iterations of the slowest chart, jumps tried, kept): the
    charts' learned runs as one batch, each chart stopped on the device at its
    own target."""
    import torch
    stream = torch.cuda.Stream()
    for c, (s, r, m), t in zip(ctxs, inputs, targets):
        c.set_stream(stream.cuda_stream)
        c.set_target_energy(t)
        c.load(s, r, m)
    b = G.Batch(ctxs)
    b.set_stream(stream.cuda_stream)
    b.set_mlp(params)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    tried, kept = b.iterate_learned(limit, jump_every)
    e1.record(stream)
    e1.synchronize()
    its = max(c.info()["iterations"] for c in ctxs)
    b.close()
    for c in ctxs:
        c.set_target_energy(0)
        c.set_stream(None)
    return e0.elapsed_time(e1) / 1e3, its, tried, kept


def time_to_energy_config(G, workload):
    """time_to_energy_line on another plain workload: plain_8192 (8192^2, 64
    Gaussians, 1,048,576 sites: the learned+batched headline configuration)
    or plain_1024 (1024^2, 8 Gaussians, 4096 sites: the learned step's
    training family, held-out seed)."""
    from workloads import config_inputs
    sites, rho, mask, _ = config_inputs(workload, seed=SEED)
    n = sites.shape[0]
    ctx = G.Context(n)
    line = time_to_energy_line(G, ctx, n, sites, rho, mask)
    ctx.close()
    line["workload"] = workload
    return line


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(values, ws, device=None):
    """The slowest replica's figures: the element-wise maximum over all ranks
    (one all-reduce; with one rank the values as they are)."""
    if ws == 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def shard_charts(weights, ws, rank):
    """The charts rank `rank` of `ws` runs: independent charts split by
    weight (pixels), largest first onto the least-loaded rank (ties to the
    lower rank), so every chart runs on exactly one rank; ascending indices."""
    load = [0] * ws
    owner = [0] * len(weights)
    for i in sorted(range(len(weights)), key=lambda i: (-weights[i], i)):
        r = min(range(ws), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += weights[i]
    return [i for i in range(len(weights)) if owner[i] == rank]


def gather_charts(mine, indices, ws, total):
    """Per-chart results of every rank, in chart order, on rank 0 (None on the
    other ranks); with one rank the list as it is.  One gather of Python
    objects (gloo or NCCL): no data-path collective, the charts are
    independent."""
    if ws == 1:
        return list(mine)
    import torch.distributed as dist
    parts = [None] * ws if dist.get_rank() == 0 else None
    dist.gather_object((list(indices), list(mine)), parts, dst=0)
    if parts is None:
        return None
    out = [None] * total
    for idx, res in parts:
        for i, r in zip(idx, res):
            out[i] = r
    return out


def job_rate(units_per_step, steps, ws, seconds):
    """Whole-job throughput in G units per second: every replica processes
    units_per_step per step, the job takes the slowest replica's seconds."""
    return units_per_step * steps * ws / seconds / 1e9


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 25 ms (a timed
    region of 10 steps lasts about 150 ms at 4096^2)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline_sample(sites, rho, mask, target_s=10.0, workload=CONFIG, iters=ITERS):
    """The oracle's OpenMP restatement of the reference's Lloyd loop (faithful
    FP32 mode, all host threads) on a bounded sample: as many iterations of
    the 4096^2 workload as fit in about target_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    n = sites.shape[0]
    t = time.perf_counter()
    orc.gcvt(sites, rho, mask, 1, 1, mode=orc.FAITHFUL, fixed_iters=1)
    t1 = time.perf_counter() - t
    k = int(max(1, min(iters, target_s / max(t1, 1e-3))))
    t = time.perf_counter()
    orc.gcvt(sites, rho, mask, 1, k, mode=orc.FAITHFUL, fixed_iters=k)
    dt = time.perf_counter() - t
    # k iterations + the final labelling pass
    value = n * n * (k + 1) / dt / 1e9
    return {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "%d Lloyd iterations + final labelling of the %s workload, faithful FP32 "
                      "restatement of gcvt.cu, %.1f s" % (k, workload, dt)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from workloads import config_inputs
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    workload = args.config if args.config in PLAIN else CONFIG
    sites, rho, mask, _ = config_inputs(workload, seed=SEED)
    n = sites.shape[0]
    iters_per_step = 2
    for _ in range(args.warmup):
        orc.gcvt(sites, rho, mask, 1, iters_per_step, mode=orc.FAITHFUL, fixed_iters=iters_per_step)
    t = time.perf_counter()
    for _ in range(args.steps):
        orc.gcvt(sites, rho, mask, 1, iters_per_step, mode=orc.FAITHFUL, fixed_iters=iters_per_step)
    dt = time.perf_counter() - t
    value = n * n * (iters_per_step + 1) * args.steps / dt / 1e9
    line = {
        "impl": "reference", "value": value, "unit": UNIT, "n_gpus": ws,
        "metric": metric_of(workload, n, int((sites[..., 0] != -32768).sum())),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+int16",
        "data": "synthetic (seeded Gaussian density on a disk, uniform sites)",
        "config": {"workload": workload, "n": n, "sites": int((sites[..., 0] != -32768).sum()),
                   "sample_iterations_per_step": iters_per_step},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": "%d Lloyd iterations + final labelling per step, faithful "
                                   "FP32 OpenMP restatement of gcvt.cu" % iters_per_step},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import gcvt_gb300 as G
    from workloads import config_inputs
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    workload = args.config if args.config in PLAIN else CONFIG
    sites, rho, mask, iters = config_inputs(workload, seed=SEED)
    passes = iters + 1
    n = sites.shape[0]
    nsites = int((sites[..., 0] != -32768).sum())
    stream = torch.cuda.Stream(device=dev)
    d_sites = torch.from_numpy(sites).to(dev)
    d_rho = torch.from_numpy(rho).to(dev)
    d_mask = torch.from_numpy(mask).to(dev)
    d_out = torch.empty_like(d_sites)
    h_sites = torch.from_numpy(sites).pin_memory()
    h_rho = torch.from_numpy(rho).pin_memory()
    h_mask = torch.from_numpy(mask).pin_memory()
    h_out = torch.empty(d_sites.shape, dtype=torch.int16).pin_memory()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > L2
    ctx = G.Context(n)
    ctx.set_stream(stream.cuda_stream)

    loop_ms = []  # iterations 2..iters of each timed device step

    def step_device(record=False):
        ctx.load(d_sites, d_rho, d_mask)
        ctx.iterate(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.iterate(iters - 1)
        b.record(stream)
        ctx.label(d_out)
        if record:
            loop_ms.append((a, b))

    def step_host():
        ctx.load(h_sites, h_rho, h_mask)
        ctx.iterate(1)
        ctx.iterate(iters - 1)
        ctx.label(h_out)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    def timed(step_fn, steps):
        total = 0.0
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_fn()
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1)
        barrier()
        return total / 1e3

    with torch.cuda.stream(stream):
        # launch choices for this workload (results do not depend on them)
        ctx.load(d_sites, d_rho, d_mask)
        ctx.iterate(3)
        tuning = ctx.autotune()
        for _ in range(args.warmup):
            step_device()
        with ClockSampler(local) as clk:
            t_dev = timed(lambda: step_device(True), args.steps)
        iter_ms = statistics.mean(a.elapsed_time(b) for a, b in loop_ms) / (iters - 1)
        info = ctx.info()  # state after the last timed step's 100 iterations
        for _ in range(max(1, args.warmup // 2)):
            step_host()
        t_e2e = timed(step_host, args.steps)
        # time to E <= (1 + 1e-4) E_conv: plain, learned, learned + batched
        tte = time_to_energy_line(G, ctx, n, sites, rho, mask)
        ctx.set_stream(stream.cuda_stream)  # the timing runs used a stream of their own
        headline = rank == 0 and not args.no_headline
        tte_8192 = (time_to_energy_config(G, "plain_8192") if headline
                    and workload != "plain_8192" else None)
        tte_1024 = (time_to_energy_config(G, "plain_1024") if headline
                    and workload != "plain_1024" else None)
        # the Delaunay triangulation of the converged sites (outside the timing)
        _, delaunay = delaunay_stage(ctx, G.load_library(), len(ctx.extract_points()), args)
        # a labelling pass (final output) and a jump-flooding labelling,
        # timed alone; the jump-flooding error on the initial sites
        ctx.load(d_sites, d_rho, d_mask)
        _, jfa_stats = ctx.jfa_label(labels=False)
        kms = ctx.time_kernels(5)
        torch.cuda.synchronize(dev)
    t_dev, t_e2e = max_over_ranks([t_dev, t_e2e], ws, dev)
    value = job_rate(n * n * passes, args.steps, ws, t_dev)
    e2e = job_rate(n * n * passes, args.steps, ws, t_e2e)
    peak, peak_kind = measured_peak()
    support_px = support_pixels(rho)
    alg = (support_px * ALG_BYTES_PER_SUPPORT_PX + n * n * ALG_BYTES_PER_PX
           + nsites * ALG_BYTES_PER_SITE)
    achieved = alg / (iter_ms / 1e3) / 1e9
    line = {
        "metric": metric_of(workload, n, nsites, iters), "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+int16",
        "data": "synthetic (seeded Gaussian density on a disk, uniform sites)",
        "config": {"workload": workload, "n": n, "sites": nsites, "iterations": iters,
                   "passes_per_step": passes, "l2": "flushed (256 MB write) before each step",
                   "parallelism": "replicas x%d" % ws},
        "iter_per_s": iters * args.steps * ws / t_dev,
        "kernel_ms": {"lloyd_iteration": iter_ms, "label_pass": kms[1], "jfa_labelling": kms[2]},
        "jfa": jfa_line(n, kms[2], jfa_stats, peak, tuning["jfa_tail_halo"]),
        "tuning": tuning,
        "time_to_energy": tte,
        "time_to_energy_8192": tte_8192,
        "time_to_energy_1024": tte_1024,
        "delaunay": delaunay,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": NCU_TRAFFIC.get(workload),
                     "peak_source": peak_kind,
                     "kernel": "k_list + k_cell<0> (one Lloyd iteration, iterations 2-100)",
                     "algorithmic_bytes": alg},
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": int(h_sites.numel() * 2 + h_rho.numel() * 4 + h_mask.numel()),
                "d2h_bytes_per_step": int(h_out.numel() * 2),
                "ms_per_step": t_e2e / args.steps * 1e3},
        # per step: load (row support, fixed bitmap, site bitmap); level
        # start (column summaries, rows, k_cover, k_cover_finish, k_count);
        # iterate(1) and iterate(ITERS - 1) as graphs of ten (k_list, k_cell)
        # pairs, launches past the last iteration returning at once; final
        # labelling (column summaries, rows)
        "gpu_launches": args.steps * (3 + 5 + 2 * 10 * (1 + (iters - 1 + 9) // 10) + 2),
        "clocks": clk.summary(),
        "final_energy": info["energy"],
    }
    if rank == 0:
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample(sites, rho, mask, workload=workload,
                                                       iters=iters)
        if not args.no_reference_gpu:
            line["reference_gpu"] = reference_gpu(sites, rho, mask, iters)
            rg = line["reference_gpu"]
            if "loop_ms" in rg:
                rg["ours_over_reference"] = rg["loop_ms"] / line["ms_per_step"]
        print(json.dumps(line))
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def reference_gpu(sites, rho, mask, iters=ITERS):
    """The reference's own kernels (compiled from its sources into
    oracle/_ref/gcvt_ref.cubin) under gcvt.cu's loop on the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    if not orc.ref_available():
        return {"unavailable": "reference cubin not built"}
    n = sites.shape[0]
    orc.ref_gcvt(sites, rho, mask, 1, 10, fixed_iters=10)
    _, info = orc.ref_gcvt(sites, rho, mask, 1, iters, fixed_iters=iters)
    return {"value": n * n * (iters + 1) / (info["loop_ms"] / 1e3) / 1e9, "unit": UNIT,
            "loop_ms": info["loop_ms"], "total_ms": info["total_ms"],
            "what": "gcvt.cu kernels on this GPU, %d iterations + final labelling; loop_ms "
                    "excludes its per-call allocation and copies, total_ms includes them" % iters}


def run_profile_case(iterations, workload=CONFIG):
    """The bench workload for ncu captures: load once, then `iterations` Lloyd
    iterations as the bench runs them (CUDA graphs of k_list + k_cell), timed
    as a whole with CUDA events on the context's stream."""
    import torch
    import gcvt_gb300 as G
    from workloads import config_inputs
    sites, rho, mask, _ = config_inputs(workload, seed=SEED)
    stream = torch.cuda.Stream()
    ctx = G.Context(sites.shape[0])
    ctx.set_stream(stream.cuda_stream)
    ctx.load(sites, rho, mask)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.iterate(iterations)
    e1.record(stream)
    e1.synchronize()
    print(json.dumps({"profile_case": workload, "iterations": iterations,
                      "lloyd_ms_per_iteration": e0.elapsed_time(e1) / iterations,
                      "energy": ctx.info()["energy"]}))
    ctx.close()
    return 0


def run_batched(args):
    """Batched uneven charts (64 charts of side 256-2048, 8 Gaussians each,
    sites = domain pixels / 64, 100 iterations): every chart loaded from HBM,
    iterated in one launch pair per iteration (gcvt_batch_iterate), labelled;
    against the same charts run one after the other (gcvt_ctx_iterate)."""
    import torch
    import gcvt_gb300 as G
    from workloads import BATCH, batched_inputs
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:  # the charts are independent: each rank runs its own share
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    all_charts = batched_inputs(seed=SEED)
    all_px = [int(s.shape[0]) ** 2 for s, _, _ in all_charts]
    mine = shard_charts(all_px, ws, rank)
    charts = [all_charts[i] for i in mine]
    stream = torch.cuda.Stream(device=dev)
    dev_in, ctxs = [], []
    for sites, rho, mask in charts:
        n = sites.shape[0]
        dev_in.append((torch.from_numpy(sites).to(dev), torch.from_numpy(rho).to(dev),
                       torch.from_numpy(mask).to(dev), torch.empty_like(torch.from_numpy(sites)).to(dev)))
        c = G.Context(n)
        c.set_stream(stream.cuda_stream)
        ctxs.append(c)
    batch = G.Batch(ctxs)
    batch.set_stream(stream.cuda_stream)
    iters = BATCH["iters"]
    px = sum(int(s.shape[0]) ** 2 for s, _, _ in charts)
    sites_total = sum(int((s[..., 0] != -32768).sum()) for s, _, _ in charts)

    def load_all():
        for c, (ds, dr, dm, _) in zip(ctxs, dev_in):
            c.load(ds, dr, dm)

    def label_all():
        for c, (_, _, _, out) in zip(ctxs, dev_in):
            c.label(out)

    def step_batched():
        load_all()
        batch.iterate(iters)
        label_all()

    def step_solo():
        load_all()
        for c in ctxs:
            c.iterate(iters)
        label_all()

    def timed(fn, steps):
        ms = []
        for _ in range(steps):
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.mean(ms)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step_batched()
        barrier()
        with ClockSampler(local) as clk:
            t_b = timed(step_batched, args.steps)
        barrier()
        energies = [c.info()["energy"] for c in ctxs]
        for _ in range(1):
            step_solo()
        t_s = timed(step_solo, max(1, args.steps // 2))
        same = all(abs(c.info()["energy"] - e) == 0.0 for c, e in zip(ctxs, energies))
    t_b, t_s, same_all = max_over_ranks([t_b, t_s, 0.0 if same else 1.0], ws, device=dev)
    per_chart = gather_charts([{"n": int(s.shape[0]), "energy": e} for (s, _, _), e in
                               zip(charts, energies)], mine, ws, len(all_charts))
    if rank != 0:
        batch.close()
        for c in ctxs:
            c.close()
        return 0
    px = sum(all_px)  # the whole job: every rank's charts
    sites_total = sum(int((s[..., 0] != -32768).sum()) for s, _, _ in all_charts)
    line = {
        "metric": "Gpix-pass/s, batched uneven charts (64 charts, side 256-2048, 100 iterations)",
        "value": px * (iters + 1) / (t_b / 1e3) / 1e9, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_b,
        "higher_is_better": True, "scaling": "strong" if ws > 1 else "weak",
        "vs_baseline": None,
        "dtype": "f32+int16", "data": "synthetic (seeded Gaussian densities on disks, uniform sites)",
        "config": {"workload": "batched_64", "charts": len(charts),
                   "sides": sorted({int(s.shape[0]) for s, _, _ in charts}),
                   "pixels": px, "sites": sites_total, "iterations": iters},
        "solo": {"ms_per_step": t_s, "value": px * (iters + 1) / (t_s / 1e3) / 1e9,
                 "what": "the same charts one after the other, gcvt_ctx_iterate each"},
        "batched_over_solo": t_s / t_b,
        "same_energies_as_solo": same_all == 0.0,
        "sharding": {"ranks": ws, "charts_per_rank": [len(shard_charts(all_px, ws, r))
                                                      for r in range(ws)],
                     "gathered_charts": sum(1 for r in per_chart if r is not None)},
        "clocks": clk.summary(),
    }
    if args.reference_gpu:  # 64 gCVT calls of the reference's kernels, one per chart
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        if orc.ref_available():
            loop = total = 0.0
            for sites, rho, mask in all_charts:
                _, info = orc.ref_gcvt(sites, rho, mask, 1, iters, fixed_iters=iters)
                loop += info["loop_ms"]
                total += info["total_ms"]
            line["reference_gpu"] = {"loop_ms": loop, "total_ms": total,
                                     "value": px * (iters + 1) / (loop / 1e3) / 1e9,
                                     "what": "the reference's gCVT kernels, one call per chart"}
    print(json.dumps(line))
    batch.close()
    for c in ctxs:
        c.close()
    return 0


def run_mesh(args):
    """Mesh-driven density (256 x 256-vertex jittered disk mesh with a height
    field, per-vertex area-ratio weights): rasterised to 2048^2 on the GPU,
    65,536 sites drawn over it and the mesh's boundary vertices as fixed
    sites (the constraint points), 100 Lloyd iterations + labels per step;
    then the constrained Delaunay triangulation and the lift."""
    import torch
    import gcvt_gb300 as G
    from workloads import disk_sites, disk_surface, mesh_constraints, mesh_inputs, raster_inputs
    torch.cuda.set_device(0)
    n, m, iters = 2048, 65536, 100
    (pts, w, tris, scale), _ = mesh_inputs(256, n, seed=2)
    uv, _, _ = disk_surface(256, seed=2)
    _, _, left, lower = raster_inputs(uv, n)
    bv, be, fx, fy = mesh_constraints(uv, tris, scale, left, lower)
    mask = np.zeros((n, n), np.uint8)
    mask[fy, fx] = 1  # generateMask (gcvt.h:141-158)
    lib = G.load_library()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    rho = G.rasterize(pts, w, tris, scale, n)  # warm-up
    d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    d_w = torch.from_numpy(np.ascontiguousarray(w)).cuda()
    d_t = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    d_rho = torch.empty((n, n), dtype=torch.float32, device="cuda")
    raster_ms = []
    for _ in range(max(3, args.steps)):
        torch.cuda.synchronize()
        ev[0].record()
        G._check(lib.gcvt_rasterize(d_pts.data_ptr(), d_w.data_ptr(), len(w), d_t.data_ptr(),
                                    len(tris), d_rho.data_ptr(), float(scale), n, G.MEM_DEVICE),
                 "gcvt_rasterize")
        ev[1].record()
        ev[1].synchronize()
        raster_ms.append(ev[0].elapsed_time(ev[1]))
    rho = d_rho.cpu().numpy()
    sites = disk_sites(n, m, 3, rho)
    sites[fy, fx, 0] = fx  # putConstrains (gcvt.h:106-122): the fixed sites
    sites[fy, fx, 1] = fy
    stream = torch.cuda.Stream()
    ctx = G.Context(n)
    ctx.set_stream(stream.cuda_stream)
    d_sites = torch.from_numpy(sites).cuda()
    d_mask = torch.from_numpy(mask).cuda()
    d_out = torch.empty_like(d_sites)

    def step():
        ctx.load(d_sites, d_rho, d_mask)
        ctx.iterate(iters)
        ctx.label(d_out)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        ms = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
    t = statistics.mean(ms)
    lift = lift_stage(ctx, n, args, constraints=(bv, be))
    ref = None
    if args.reference_gpu:  # the reference's rasteriser and gCVT kernels on this mesh
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        if orc.ref_available():
            # the reference tests every triangle at every pixel: timed on the
            # 64^2-vertex mesh (its cost grows with the triangle count) and
            # scaled to this one
            (p64, w64, t64, s64), _ = mesh_inputs(64, n, seed=2)
            ref_rho, ref_ms = orc.ref_rasterize(p64, w64, t64, s64, n)
            ours64 = G.rasterize(p64, w64, t64, s64, n)
            _, info = orc.ref_gcvt(sites, rho, mask, 1, iters, fixed_iters=iters)
            ref = {"raster_ms_64": ref_ms, "triangles_64": int(len(t64)),
                   "raster_ms_scaled": ref_ms * len(tris) / len(t64),
                   "same_density_64": bool(np.array_equal(ref_rho.view(np.int32),
                                                          ours64.view(np.int32))),
                   "loop_ms": info["loop_ms"], "total_ms": info["total_ms"]}
    print(json.dumps({
        "metric": "Gpix-pass/s, mesh-driven density (2048^2 raster of a 256^2-vertex disk mesh), 65,536 sites, 100 iterations",
        "value": n * n * (iters + 1) / (t / 1e3) / 1e9, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 raster, f32+int16 Lloyd",
        "data": "synthetic (seeded jittered disk mesh, height field, area-ratio weights)",
        "config": {"workload": "mesh_2048", "n": n, "triangles": int(len(tris)),
                   "vertices": int(len(w)), "sites": m, "fixed_sites": int(mask.sum()),
                   "constraint_segments": int(len(be)), "iterations": iters},
        "raster_ms": statistics.median(raster_ms),
        "lift": lift,
        "reference_gpu": ref,
        "final_energy": ctx.info()["energy"]}))
    ctx.close()
    return 0


def delaunay_stage(ctx, lib, npts, args):
    """The Delaunay triangulation of the final sites on the GPU
    (gcvt_ctx_delaunay, device output; the call is host-synchronous, so it is
    timed on the host clock), and scipy's Qhull on the same points on the
    host for comparison (a library, not the reference: the reference's
    gDel2D does not build here)."""
    import ctypes
    import torch
    import gcvt_gb300 as G
    cap = max(2 * npts - 5, 1)
    d_tri = torch.empty((cap, 3), dtype=torch.int32, device="cuda")
    cnt = ctypes.c_int(0)
    times = []
    for r in range(max(3, args.warmup) + max(3, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        G._check(lib.gcvt_ctx_delaunay(ctx.h, d_tri.data_ptr(), cap, ctypes.byref(cnt),
                                       G.MEM_DEVICE), "gcvt_ctx_delaunay")
        if r >= max(3, args.warmup):
            times.append((time.perf_counter() - t0) * 1e3)
    res = {"triangles": int(cnt.value), "ms": statistics.median(times)}
    try:
        from scipy.spatial import Delaunay
        pts = ctx.extract_points()
        t0 = time.perf_counter()
        q = Delaunay(pts)
        res["qhull_ms"] = (time.perf_counter() - t0) * 1e3
        res["qhull_triangles"] = int(len(q.simplices))
    except ImportError:
        pass
    return d_tri[:cnt.value], res


def cdt_stage(ctx, lib, scale, left, lower, cpts, segs, args):
    """The constrained Delaunay triangulation of the final free sites and the
    constraint points with the constraint segments (gcvt_ctx_cdt, device
    output; host-synchronous, so timed on the host clock)."""
    import ctypes
    import torch
    import gcvt_gb300 as G
    F = len(ctx.extract_points())
    cap = 2 * (F + len(cpts)) + 16
    d_tri = torch.empty((cap, 3), dtype=torch.int32, device="cuda")
    d_c = torch.from_numpy(np.ascontiguousarray(cpts, np.float64)).cuda()
    d_s = torch.from_numpy(np.ascontiguousarray(segs, np.int32)).cuda()
    cnt, det = ctypes.c_int(0), ctypes.c_int(0)
    times = []
    for r in range(max(3, args.warmup) + max(3, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        G._check(lib.gcvt_ctx_cdt(ctx.h, float(scale), float(left), float(lower), d_c.data_ptr(),
                                  len(cpts), d_s.data_ptr(), len(segs), d_tri.data_ptr(), cap,
                                  ctypes.byref(cnt), ctypes.byref(det), G.MEM_DEVICE),
                 "gcvt_ctx_cdt")
        if r >= max(3, args.warmup):
            times.append((time.perf_counter() - t0) * 1e3)
    return d_tri[:cnt.value], {"triangles": int(cnt.value), "ms": statistics.median(times),
                               "free_sites": F, "constraint_points": int(len(cpts)),
                               "segments": int(len(segs))}


def lift_stage(ctx, n, args, constraints=None):
    """The stages after the Lloyd loop: the final sites, extracted as CDT
    input points (delaunay.h:46-57), triangulated on the GPU -- with the
    constraint points and segments (bv, be: boundary vertices and edges of
    the mesh) by gcvt_ctx_cdt, else gcvt_ctx_delaunay -- lifted onto the
    surface and the triangles filtered (recover.h:98-157) by gcvt_lift,
    device buffers, CUDA events.  Beside it, the oracle's single-thread
    restatement of recover() -- the reference's O(queries x faces) scan --
    timed on 400 queries and scaled to all."""
    import torch
    import gcvt_gb300 as G
    from workloads import disk_surface, raster_inputs
    uv, xyz, tris = disk_surface(256, seed=2)
    _, scale, left, lower = raster_inputs(uv, n)
    pts = ctx.extract_points(scale, left, lower)
    lib = G.load_library()
    fixed = np.zeros(0, np.int32)
    if constraints is not None:
        bv, be = constraints
        F = len(pts)
        pos = {int(v): k for k, v in enumerate(bv)}
        segs = np.array([(F + pos[int(a)], F + pos[int(b)]) for a, b in be], np.int32)
        d_cdt, dstage = cdt_stage(ctx, lib, scale, left, lower, uv[bv], segs, args)
        pts = np.concatenate([pts, uv[bv]])
        fixed = np.ascontiguousarray(bv, np.int32)
    else:
        d_cdt, dstage = delaunay_stage(ctx, lib, len(pts), args)
    cdt = d_cdt.cpu().numpy()
    d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (uv, xyz, tris, pts)] + [d_cdt]
    d_fix = torch.from_numpy(fixed).cuda() if len(fixed) else None
    out = torch.empty((len(pts), 3), dtype=torch.float64, device="cuda")
    face = torch.empty(len(pts), dtype=torch.int32, device="cuda")
    keep = torch.empty(len(cdt), dtype=torch.uint8, device="cuda")

    def call():
        G._check(lib.gcvt_lift(d[0].data_ptr(), d[1].data_ptr(), len(uv), d[2].data_ptr(),
                               len(tris), d[3].data_ptr(), len(pts), len(fixed),
                               None if d_fix is None else d_fix.data_ptr(), d[4].data_ptr(),
                               len(cdt), out.data_ptr(), face.data_ptr(), keep.data_ptr(),
                               G.MEM_DEVICE), "gcvt_lift")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    times = []
    for r in range(max(3, args.warmup) + max(3, args.steps)):
        torch.cuda.synchronize()
        ev[0].record()
        call()
        ev[1].record()
        ev[1].synchronize()
        if r >= max(3, args.warmup):
            times.append(ev[0].elapsed_time(ev[1]))
    res = {"points": int(len(pts)), "faces": int(len(tris)), "cdt_triangles": int(len(cdt)),
           "kept": int(keep.sum().item()), "located": int((face >= 0).sum().item()),
           "lift_ms": statistics.median(times),
           ("cdt" if constraints is not None else "delaunay"): dstage}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        rng = np.random.default_rng(0)
        sp = pts[rng.choice(len(pts), 200, replace=False)]
        corners = pts[cdt[rng.choice(len(cdt), 200, replace=False)]].reshape(-1, 2)
        t0 = time.perf_counter()
        orc.lift(uv, xyz, tris, sp, threads=1)
        t1 = time.perf_counter()
        # the corners as constraint points (not located), their triangles' centroids located
        orc.lift(uv, xyz, tris, corners, np.zeros(600, np.int32),
                 np.arange(600, dtype=np.int32).reshape(200, 3), threads=1)
        t2 = time.perf_counter()
        res["cpu_baseline"] = {"kind": "port", "cores": 1,
                               "sample": "200 points and 200 triangles, scaled to all",
                               "ms": ((t1 - t0) * len(pts) + (t2 - t1) * len(cdt)) / 200 * 1e3}
    return res


def run_profile_lift(repeats):
    """gcvt_lift alone, `repeats` times (for ncu): 65,536 points uniform in the
    disk on the 256^2-vertex disk mesh, scipy's Delaunay of them as the CDT."""
    import torch
    import gcvt_gb300 as G
    from scipy.spatial import Delaunay
    from workloads import disk_surface
    uv, xyz, tris = disk_surface(256, seed=2)
    rng = np.random.default_rng(5)
    r = 0.47 * np.sqrt(rng.random(65536))
    a = rng.random(65536) * 2 * np.pi
    pts = np.stack([0.5 + r * np.cos(a), 0.5 + r * np.sin(a)], 1)
    cdt = Delaunay(pts).simplices.astype(np.int32)
    lib = G.load_library()
    d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (uv, xyz, tris, pts, cdt)]
    out = torch.empty((len(pts), 3), dtype=torch.float64, device="cuda")
    face = torch.empty(len(pts), dtype=torch.int32, device="cuda")
    keep = torch.empty(len(cdt), dtype=torch.uint8, device="cuda")
    ms = []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for _ in range(repeats):
        torch.cuda.synchronize()
        ev[0].record()
        G._check(lib.gcvt_lift(d[0].data_ptr(), d[1].data_ptr(), len(uv), d[2].data_ptr(),
                               len(tris), d[3].data_ptr(), len(pts), 0, None, d[4].data_ptr(),
                               len(cdt), out.data_ptr(), face.data_ptr(), keep.data_ptr(),
                               G.MEM_DEVICE), "gcvt_lift")
        ev[1].record()
        ev[1].synchronize()
        ms.append(ev[0].elapsed_time(ev[1]))
    print(json.dumps({"profile_lift": {"points": len(pts), "faces": len(tris),
                                       "triangles": len(cdt)}, "ms": ms}))
    return 0


def run_profile_delaunay(repeats, workload):
    """The Delaunay of a plain workload's sites after its Lloyd iterations,
    `repeats` times into a device buffer (for ncu)."""
    import ctypes
    import torch
    import gcvt_gb300 as G
    from workloads import config_inputs
    sites, rho, mask, iters = config_inputs(workload, seed=SEED)
    ctx = G.Context(sites.shape[0])
    ctx.load(sites, rho, mask)
    ctx.iterate(iters)
    cap = 2 * len(ctx.extract_points())
    d = torch.empty((cap, 3), dtype=torch.int32, device="cuda")
    cnt = ctypes.c_int(0)
    lib = G.load_library()
    ms = []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        G._check(lib.gcvt_ctx_delaunay(ctx.h, d.data_ptr(), cap, ctypes.byref(cnt), G.MEM_DEVICE),
                 "gcvt_ctx_delaunay")
        ms.append((time.perf_counter() - t0) * 1e3)
    print(json.dumps({"profile_delaunay": workload, "iterations": iters,
                      "triangles": cnt.value, "ms": ms}))
    ctx.close()
    return 0


def run_profile_jfa(repeats):
    """The bench workload's jump-flooding labelling, `repeats` times (for ncu)."""
    import torch
    import gcvt_gb300 as G
    from workloads import config_inputs
    sites, rho, mask, _ = config_inputs(CONFIG, seed=SEED)
    ctx = G.Context(sites.shape[0])
    ctx.load(sites, rho, mask)
    ms = ctx.time_kernels(repeats)[2]
    torch.cuda.synchronize()
    print(json.dumps({"profile_jfa": CONFIG, "repeats": repeats, "jfa_ms": ms}))
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-gpu", action="store_true",
                    help="batched_64: also time the reference's own kernels on this GPU")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="plain workloads: skip timing the reference's own kernels on this GPU")
    ap.add_argument("--no-headline", action="store_true",
                    help="skip the 8192^2 time-to-energy line (plain vs learned vs learned+batched)")
    ap.add_argument("--profile-case", type=int, default=0, metavar="ITERS",
                    help="only run ITERS Lloyd iterations of the workload (for ncu)")
    ap.add_argument("--config", default=CONFIG,
                    choices=list(PLAIN) + ["batched_64", "mesh_2048"],
                    help="batched_64 / mesh_2048: the batched-charts or mesh-driven workload "
                         "(their own JSON lines)")
    ap.add_argument("--profile-jfa", type=int, default=0, metavar="REPEATS",
                    help="only run REPEATS jump-flooding labellings of the workload (for ncu)")
    ap.add_argument("--profile-lift", type=int, default=0, metavar="REPEATS",
                    help="only run REPEATS lifts of 65,536 points on the mesh (for ncu)")
    ap.add_argument("--profile-delaunay", type=int, default=0, metavar="REPEATS",
                    help="only run REPEATS Delaunay triangulations of the workload's sites "
                         "after its Lloyd iterations (for ncu)")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args.profile_case,
                                args.config if args.config in PLAIN else CONFIG)
    if args.profile_jfa:
        return run_profile_jfa(args.profile_jfa)
    if args.profile_lift:
        return run_profile_lift(args.profile_lift)
    if args.profile_delaunay:
        return run_profile_delaunay(args.profile_delaunay,
                                    args.config if args.config in PLAIN else CONFIG)
    if args.warmup < 3:
        args.warmup = 3
    if args.config == "batched_64" and args.impl == "ours":
        return run_batched(args)
    if args.config == "mesh_2048" and args.impl == "ours":
        return run_mesh(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
