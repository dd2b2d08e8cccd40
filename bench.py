"""Benchmark of the GB300-native TUCuda filter path.

Workload (the batched configuration): 256 images, widths U[320,4096], heights
U[240,2160], FP16 storage of U[0,255) pixels, each drawing one operator from
{Gaussian smooth sigma 1, 2, 4, 8; box radius 3, 7, 15 (window means)}, run as
ONE CUDA-graph launch (one concurrent kernel per operator class).  A step is one
pass over the whole batch.  Inputs (1.36 GB) exceed L2 (129 MB), so no flush is needed
between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--only-batch]

Prints one JSON line.  --impl reference times the CPU restatement of the
reference's arithmetic (oracle/, the reference's own CPU filters live in the
absent TULibs library) on the host cores, on a bounded sample of the same
workload.  Under torchrun every rank runs the same batch (weak scaling, no
collective on the data path); rank 0 prints.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpix/s"
E2E_CHUNKS = 32  # groups of the end-to-end run (copies overlap kernels)
# Serving traces (req/s, requests): the configured 100k-request trace at 10k and
# 20k req/s, and the first 10k requests at 2k req/s (5 s of arrivals).
SERVING_RUNS = ((2000.0, 10000), (10000.0, 100000), (20000.0, 100000))
CPU_SAMPLE_MPIX = 256.0  # CPU restatement sample (main line's cpu_baseline and the reference arm)
WORKLOAD = ("batched: 256 images W~U[320,4096] H~U[240,2160], FP16 storage of U[0,255), "
            "ops {Gaussian smooth sigma 1,2,4,8; box mean radius 3,7,15}, one CUDA-graph "
            "launch per step (tensor-core path: one kernel for every job)")
ARITHMETIC = ("tensor cores (tcgen05 kind::f16): f16 pixels, taps and horizontal results as "
              "f16 hi/lo pairs, FP32 accumulation in tensor memory")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the batched kernel from the committed ncu
    summary (profiles/fir_tc_kernel_batched_f16.md), or None."""
    path = os.path.join(ROOT, "profiles", "fir_tc_kernel_batched_f16.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


# ---- distributed plumbing ---------------------------------------------------------

def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world, local


def barrier(world):
    from tucuda_gb300 import replicas
    replicas.barrier()


def max_over_ranks(x, world):
    from tucuda_gb300 import replicas
    return replicas.max_over_ranks(x)


# ---- clocks ---------------------------------------------------------------------------

class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""
        return False

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---- the batched workload ----------------------------------------------------------

def build_workload(dev, storage="f16", rank=0, world=1):
    """The batched workload's images; with world > 1 only this rank's share
    (replicas.shard: a deterministic longest-first split by pixel count, the
    same on every rank, no data exchanged)."""
    import torch
    from tucuda_gb300 import replicas, workloads

    jobs = workloads.batched_spec(seed=4, n=256, dtype=storage)
    if world > 1:
        mine = replicas.shard([j.rows * j.cols for j in jobs], rank, world)
        jobs = [jobs[i] for i in mine]
    dt = {"f16": torch.float16, "f32": torch.float32, "u8": torch.uint8}[storage]
    es = torch.empty((), dtype=dt).element_size()
    # One packed device buffer for all inputs and one for all outputs (rows
    # padded to 128 bytes, images 256-byte aligned), so that the end-to-end
    # run moves each direction with a single copy.
    layout, off = [], 0
    for j in jobs:
        pitch = (j.cols * es + 127) // 128 * 128
        layout.append((off, pitch))
        off += (pitch * j.rows + 255) // 256 * 256
    total = off
    inbuf = torch.empty(total // es, dtype=dt, device=dev)
    outbuf = torch.zeros(total // es, dtype=dt, device=dev)
    ins, outs = [], []
    for j, (o, pitch) in zip(jobs, layout):
        pe = pitch // es
        v = inbuf[o // es:o // es + pe * j.rows].view(j.rows, pe)[:, :j.cols]
        workloads.fill_uniform_(v, j.seed)
        ins.append(v)
        outs.append(outbuf[o // es:o // es + pe * j.rows].view(j.rows, pe)[:, :j.cols])
    return jobs, ins, outs, inbuf, outbuf


def add_jobs(batch, jobs, ins, outs):
    for j, a, b in zip(jobs, ins, outs):
        if j.op == "gauss":
            batch.add_gauss(a, b, j.sigma)
        else:
            batch.add_box(a, b, j.window, j.window, normalize=True)


def plain_pass(jobs, ins, outs, tensor=False, cache=None):
    """One pass of per-image launches (the single-image path); tensor=True
    with the handles' tensor-core switch on."""
    from tucuda_gb300 import filters as F
    gs, bs = ({}, {}) if cache is None else cache
    for j, a, b in zip(jobs, ins, outs):
        if j.op == "gauss":
            g = gs.get(j.sigma)
            if g is None:
                g = gs[j.sigma] = F.FIRGaussianConvolver2(j.sigma).set_tensor_cores(tensor)
            g.smooth(a, b)
        else:
            f = bs.get(j.window)
            if f is None:
                f = bs[j.window] = F.BoxFilter2(j.window, j.window, 64).set_tensor_cores(tensor)
            f.convolve(a, b, True, True)


def time_events(fn, reps):
    import torch
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


# ---- CPU baseline (the oracle restatement) ----------------------------------------------

def cpu_prepare(min_mpix, seed=4):
    """Inputs for the CPU baseline: images of the batched workload (FP16-rounded
    U[0,255) values, as float32), taken one operator kind at a time in turn
    (the workload draws its seven kinds uniformly) until every kind is present
    and `min_mpix` megapixels are reached."""
    from tucuda_gb300 import workloads
    jobs = workloads.batched_spec(seed=seed, n=256)
    rng = np.random.default_rng(seed)
    imgs = [(rng.random((j.rows, j.cols), dtype=np.float32) * 255).astype(np.float16) for j in jobs]
    kinds = {}
    for j, img in zip(jobs, imgs):
        kinds.setdefault((j.op, j.sigma, j.radius), []).append((j, img))
    queues = list(kinds.values())
    sample, px, k = [], 0, 0
    while any(queues):
        q = queues[k % len(queues)]
        k += 1
        if not q:
            continue
        j, img = q.pop(0)
        sample.append((j, img.astype(np.float32)))
        px += j.pixels
        if px >= min_mpix * 1e6 and k >= len(queues):
            break
    return sample, px


def cpu_time(sample):
    """Seconds the CPU restatement takes over the sample (all host threads)."""
    from oracle import oracle as orc
    lobes = {}
    t0 = time.perf_counter()
    for j, img in sample:
        if j.op == "gauss":
            l0 = lobes.setdefault(j.sigma, orc.gauss_lobes(j.sigma)[0])
            orc.fir_f32(img, l0, l0)
        else:
            orc.box_f32(img, j.window, j.window)
    return time.perf_counter() - t0


def precision_report(jobs, ins, outs):
    """Max and relative RMS error of the batched FP16-storage outputs against
    the FP64 oracle (FP64-designed Gaussian lobes, FP64 window means, both over
    the stored FP16 inputs), per operator kind, on the smallest image of each
    kind in the workload."""
    from oracle import oracle as orc
    from tucuda_gb300 import workloads
    pick = {}
    for i, j in enumerate(jobs):
        key = (j.op, j.sigma if j.op == "gauss" else j.window)
        if key not in pick or j.pixels < jobs[pick[key]].pixels:
            pick[key] = i
    rows_out = []
    for (op, arg), i in sorted(pick.items()):
        j = jobs[i]
        x = ins[i].float().cpu().numpy().astype(np.float64)
        y = outs[i].float().cpu().numpy().astype(np.float64)
        if op == "gauss":
            l0 = orc.gauss_lobes_f64(arg)[0]
            _, ref = orc.fir_f64(x, l0, l0)
            ls = len(l0) & ~1
            v = (slice(ls, j.rows - ls), slice(ls, j.cols - ls))
            name = f"Gaussian smooth sigma {arg:g}"
        else:
            _, ref = orc.box_f64(x, arg, arg)
            ref = ref / (arg * arg)
            h = arg // 2
            v = (slice(h, h + j.rows + 1 - arg), slice(h, h + j.cols + 1 - arg))
            name = f"box mean {arg}x{arg}"
        d = y[v] - ref[v]
        rows_out.append({"output": name, "image": f"{j.cols}x{j.rows}",
                         "max_abs": round(float(np.abs(d).max()), 5),
                         "rel_rms": float(f"{np.sqrt(np.mean(d * d)) / np.sqrt(np.mean(ref[v] ** 2)):.3g}")})
    # FP32 storage (no output rounding): configurations 1 and 3 against FP64
    import torch
    from tucuda_gb300 import filters as F
    dev = ins[0].device
    fp32 = []
    img = workloads.plain_image()
    g = F.FIRGaussianConvolver2(2.0)
    out = torch.zeros(img.shape, dtype=torch.float32, device=dev)
    g.smooth(torch.from_numpy(img).to(dev), out)
    l0 = orc.gauss_lobes_f64(2.0)[0]
    _, ref = orc.fir_f64(img.astype(np.float64), l0, l0)
    ls = len(l0) & ~1
    v = (slice(ls, img.shape[0] - ls), slice(ls, img.shape[1] - ls))
    fp32.append(_err("Gaussian smooth sigma 2, 640x480 f32", out.cpu().numpy()[v], ref[v]))
    p, gd = workloads.guided_pair()
    go = torch.zeros(p.shape, dtype=torch.float32, device=dev)
    F.GuidedFilter2(17, 17, workloads.GUIDED_E, 23).convolve(torch.from_numpy(p).to(dev),
                                                              torch.from_numpy(gd).to(dev), go)
    _, gref = orc.guided_f64(p, gd, 17, 17, workloads.GUIDED_E)
    v = (slice(16, p.shape[0] - 16), slice(16, p.shape[1] - 16))
    fp32.append(_err("guided filter r8, 1920x1080 f32", go.cpu().numpy()[v], gref[v]))
    return {"vs": "FP64 oracle over the stored inputs (values 0..255)", "storage": "f16",
            "bar_rel_rms": 1e-3, "max_rel_rms": max(r["rel_rms"] for r in rows_out),
            "per_output": rows_out, "fp32_storage": fp32}


def _err(name, got, ref):
    d = got.astype(np.float64) - ref
    return {"output": name, "max_abs": float(f"{np.abs(d).max():.3g}"),
            "rel_rms": float(f"{np.sqrt(np.mean(d * d)) / np.sqrt(np.mean(ref ** 2)):.3g}")}


def cpu_extrema():
    """The oracle's restatement of the extrema_finder deque passes over the
    three 1920x1080 u8 planes (15x15 minima and positions), all host threads."""
    from oracle import oracle as orc
    from tucuda_gb300 import workloads
    planes = workloads.planes_u8().astype(np.float64)
    orc.extrema(planes[0], 15, 15)
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        for k in range(planes.shape[0]):
            orc.extrema(planes[k], 15, 15)
    secs = (time.perf_counter() - t0) / reps
    return {"gpix_per_s": round(planes.size / secs / 1e9, 4), "threads": orc.max_threads(),
            "kind": "port (deque restatement, oracle/tucu_oracle.c)"}


def cpu_features():
    """The oracle's FP32 box filter over each of the four feature channels
    (the restatement of box_convolver on vec<float, 4>), all host threads."""
    from oracle import oracle as orc
    from tucuda_gb300 import workloads
    feat = workloads.feature_image()
    chans = [np.ascontiguousarray(feat[:, :, c]) for c in range(feat.shape[2])]
    t0 = time.perf_counter()
    for ch in chans:
        orc.box_f32(ch, 15, 15)
    secs = time.perf_counter() - t0
    return {"gpix_per_s": round(feat.shape[0] * feat.shape[1] / secs / 1e9, 4),
            "threads": orc.max_threads(), "kind": "port (oracle/tucu_oracle.c, per channel)"}


def cpu_stereo():
    """The oracle's stereo cost aggregation on the same image pair, 16 of the
    64 disparities (the rate per cost value does not depend on how many)."""
    from oracle import oracle as orc
    from tucuda_gb300 import workloads
    left, right = (a.astype(np.float64) for a in workloads.stereo_pair())
    t0 = time.perf_counter()
    orc.stereo(left, right, 7, 7, 50, 16)
    secs = time.perf_counter() - t0
    return {"gcost_per_s": round(left.size * 16 / secs / 1e9, 4), "threads": orc.max_threads(),
            "kind": "port (oracle/tucu_oracle.c, 16 disparities)"}


def cpu_select():
    """The oracle's disparity selection over a 64-disparity volume of 270 rows
    of the stereo pair's size (the rate per pixel does not depend on the row
    count)."""
    from oracle import oracle as orc
    rng = np.random.default_rng(1)
    vol = rng.integers(0, 2000, (64, 270, 1914)).astype(np.float64)
    t0 = time.perf_counter()
    orc.select_disparity(vol, 80, 2)
    secs = time.perf_counter() - t0
    return {"gpix_per_s": round(270 * 1914 / secs / 1e9, 4), "threads": orc.max_threads(),
            "kind": "port (oracle/tucu_oracle.c)"}


def cpu_desc(sample, px):
    from oracle import oracle as orc
    return (f"{len(sample)} images of the batched workload, every operator kind ({px / 1e6:.1f} Mpix), FP32 C "
            f"restatement of the reference arithmetic (oracle/tucu_oracle.c), OpenMP "
            f"{orc.max_threads()} threads"), orc.max_threads()


def run_reference(args, rank, world):
    if rank != 0:
        return
    # the same sample as the main line's cpu_baseline, one pass per step
    sample, px = cpu_prepare(CPU_SAMPLE_MPIX)
    desc, threads = cpu_desc(sample, px)
    for _ in range(args.warmup):
        cpu_time(sample)
    secs = [cpu_time(sample) for _ in range(args.steps)]
    value = px * len(secs) / sum(secs) / 1e9
    line = {"metric": METRIC, "value": round(value, 4), "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sum(secs) / len(secs), 2),
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample_per_step": desc},
            "cpu_baseline": {"value": round(value, 4), "unit": METRIC, "cores": threads,
                             "kind": "port", "sample": desc},
            "e2e": {"value": round(value, 4), "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- serving (configuration 5, reduced trace) ------------------------------------------

def run_serving(n=2000, rate=10000.0, budget=32 << 30, seed=5, streams=6, max_wave=16, ring_slots=192):
    """Replays the first n requests of the serving trace (Poisson arrivals at
    `rate` req/s; sizes log-uniform 640x480..3840x2160; u8/f16 50/50; 50%
    Gaussian smooth, 30% box means, 20% guided) through the server with host
    images in pinned memory; returns latency and throughput figures."""
    import torch
    from tucuda_gb300 import workloads
    from tucuda_gb300.server import Server
    trace = workloads.serving_trace(seed=seed, n=n, rate=rate)
    maxr, maxc = 2160, 3840
    pool = {}
    for dt, tdt in (("u8", torch.uint8), ("f16", torch.float16)):
        imgs = []
        for k in range(4):
            t = torch.empty(maxr, maxc, dtype=tdt, pin_memory=True)
            workloads.fill_uniform_(t, seed * 10 + k)
            imgs.append(t)
        pool[dt] = imgs
    ring = [torch.empty(maxr, maxc, dtype=torch.float16, pin_memory=True) for _ in range(ring_slots)]
    owner = [None] * len(ring)
    tickets = []

    def submit(srv, j, src, dst):
        if j.op == "gauss":
            return srv.submit_gauss(src, dst, j.sigma)
        if j.op == "box":
            return srv.submit_box(src, dst, j.radius, normalize=True)
        return srv.submit_guided(src, None, dst, j.radius, workloads.GUIDED_E)

    # Untimed warm-up through a throwaway server: one request of every kind in
    # the trace, so that one-time costs (first launches of each kernel, lazy
    # module loading) stay out of the measured latencies.
    kinds = {}
    for j in trace:
        kinds.setdefault((j.op, j.dtype, round(j.sigma) if j.op == "gauss" else j.radius), j)
    with Server(budget_bytes=1 << 30, streams=streams, max_wave=max_wave, tensor=True) as warm:
        for k, j in enumerate(kinds.values()):
            warm.wait(submit(warm, j, pool[j.dtype][0][:240, :320], ring[k % len(ring)][:240, :320]))
    with Server(budget_bytes=budget, streams=streams, max_wave=max_wave, tensor=True) as srv:
        t0 = time.perf_counter()
        for i, j in enumerate(trace):
            slot = i % len(ring)
            if owner[slot] is not None:
                srv.wait(owner[slot])
            while time.perf_counter() - t0 < j.arrival:
                pass
            t = submit(srv, j, pool[j.dtype][i % 4][:j.rows, :j.cols], ring[slot][:j.rows, :j.cols])
            owner[slot] = t
            tickets.append(t)
        for t in owner:
            if t is not None:
                srv.wait(t)
        st = srv.stats()
    return {"requests": n, "arrival_rate_per_s": rate, "p50_ms": round(st["p50_ms"], 3),
            "p99_ms": round(st["p99_ms"], 3), "gpix_per_s": round(st["gpix_per_s"], 3),
            "waves": st["waves"], "mean_wave_requests": round(st["mean_wave_requests"], 2),
            "budget_gb": budget / 2**30, "peak_gb": round(st["peak_bytes"] / 2**30, 3),
            "completed": st["completed"], "failed": st["failed"],
            "note": "host images in pinned memory; latency = submit to completion incl. copies; "
                    "one untimed request of each kind first (throwaway server)"}


# ---- configurations 1-3 (single-image path) -------------------------------------------------

def _cpu_rate(fn, px, min_s=0.5, max_reps=20):
    """Gpix/s of the CPU restatement (oracle/, all host threads): one untimed
    call, then repetitions until min_s seconds."""
    fn()
    n, t0 = 0, time.perf_counter()
    while n < 1 or (time.perf_counter() - t0 < min_s and n < max_reps):
        fn()
        n += 1
    return round(px * n / (time.perf_counter() - t0) / 1e9, 4)


def _e2e(fn, h_ins, d_ins, d_outs, h_outs, px, reps=10):
    """The same call end to end through the public API: each repetition copies
    the inputs in from pinned host memory, filters, and copies the outputs
    back, all inside the CUDA-event timed region."""
    def step():
        for h, d in zip(h_ins, d_ins):
            d.copy_(h, non_blocking=True)
        fn()
        for d, h in zip(d_outs, h_outs):
            h.copy_(d, non_blocking=True)
    step()
    ms = time_events(step, reps)
    return {"gpix_per_s": round(px / (ms * 1e-3) / 1e9, 3), "ms": round(ms, 4),
            "h2d_bytes": int(sum(t.numel() * t.element_size() for t in h_ins)),
            "d2h_bytes": int(sum(t.numel() * t.element_size() for t in h_outs))}


def _pinned(t):
    import torch
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h


def run_configs(dev, peak):
    """Configurations 1-3 on their own seeded inputs: device-resident Gpix/s
    and fraction of the measured HBM peak (CUDA events over 20 repetitions
    after warm-up), the same calls end to end with host buffers, the CPU
    restatement's Gpix/s (all host threads), and per-output max / relative RMS
    error against the FP64 oracle."""
    import torch
    from oracle import oracle as orc
    from tucuda_gb300 import filters as F
    from tucuda_gb300 import workloads
    from tucuda_gb300.batch import Batch
    res = {}
    threads = orc.max_threads()

    def rec(name, fn, px, nbytes, **extra):
        fn()
        ms = time_events(fn, 20)
        res[name] = {"gpix_per_s": round(px / (ms * 1e-3) / 1e9, 2), "ms": round(ms, 4),
                     "hbm_frac": round(nbytes / (ms * 1e-3) / 1e9 / peak, 4), **extra}
        return res[name]

    def valid(shape, ry, rx):
        return (slice(ry, shape[0] - ry), slice(rx, shape[1] - rx))

    # 1: plain Gaussian smooth, sigma 2, one 640x480 float32 image
    img_np = workloads.plain_image()
    img = torch.from_numpy(img_np).to(dev)
    out = torch.empty_like(img)
    g2 = F.FIRGaussianConvolver2(2.0)
    r = rec("1_smooth_sigma2_640x480_f32", lambda: g2.smooth(img, out), img.numel(), 8 * img.numel())
    r["e2e"] = _e2e(lambda: g2.smooth(img, out), [_pinned(img)], [img], [out], [_pinned(out)], img.numel(), 50)
    l0 = g2.lobes()[0]
    r["cpu"] = {"gpix_per_s": _cpu_rate(lambda: orc.fir_f32(img_np, l0, l0), img.numel()),
                "threads": threads, "kind": "FP32 C restatement (oracle/)"}
    d0 = orc.gauss_lobes_f64(2.0)[0]
    _, ref = orc.fir_f64(img_np.astype(np.float64), d0, d0)
    g2.smooth(img, out)
    v = valid(img_np.shape, 8, 8)
    r["errors_vs_fp64"] = [_err("smooth", out.cpu().numpy()[v], ref[v])]

    # 2a: 15x15 box sums of three 1920x1080 u8 planes -> int32, as three calls
    # and as one batched graph launch
    planes_np = workloads.planes_u8()
    planes = torch.from_numpy(planes_np).to(dev)
    sums = torch.empty(planes.shape, dtype=torch.int32, device=dev)
    box = F.BoxFilter2(15, 15, 23)

    def box3():
        for k in range(3):
            box.convolve(planes[k], sums[k])
    r = rec("2a_box15_3x1920x1080_u8_i32", box3, planes.numel(), 5 * planes.numel())
    b3 = Batch()
    for k in range(3):
        b3.add_box(planes[k], sums[k], 15, 15)
    b3.plan()
    b3.launch()
    r["batched_one_launch"] = dict(rec("_tmp", b3.launch, planes.numel(), 5 * planes.numel()))
    del res["_tmp"]
    r["e2e"] = _e2e(b3.launch, [_pinned(planes)], [planes], [sums], [_pinned(sums)], planes.numel(), 20)
    r["cpu"] = {"gpix_per_s": _cpu_rate(lambda: [orc.box_i64(planes_np[k], 15, 15) for k in range(3)],
                                        planes.numel()),
                "threads": threads, "kind": "exact int64 C restatement (oracle/)"}
    torch.cuda.synchronize()
    b3.launch()
    got = sums.cpu().numpy()
    exact = all(np.array_equal(got[k][7:7 + 1066, 7:7 + 1906].astype(np.int64),
                               orc.box_i64(planes_np[k], 15, 15)[1][7:7 + 1066, 7:7 + 1906]) for k in range(3))
    r["errors_vs_exact"] = {"bit_exact_int32": bool(exact)}

    # next row (BoxFilter2 with extrema_finder): 15x15 window minima of the
    # same planes, values (u8) and (x, y) positions (2 x int32)
    ext = F.ExtremaFilter2(15, 15, 23)
    mins = torch.empty_like(planes)
    where = torch.empty(planes.shape + (2,), dtype=torch.int32, device=dev)

    def ext3():
        for k in range(3):
            ext.convolve(planes[k], mins[k], where[k])

    def ext3v():
        for k in range(3):
            ext.convolve(planes[k], mins[k])
    rec("next_extrema_min15_3x1920x1080_u8_val_pos", ext3, planes.numel(), 10 * planes.numel())
    rec("next_extrema_min15_3x1920x1080_u8_val", ext3v, planes.numel(), 2 * planes.numel())
    # 2b: the six Gaussian operators at sigma 3 in one pass, f32 and f16 storage
    g3 = F.FIRGaussianConvolver2(3.0)
    lob = g3.lobes()
    lob64 = orc.gauss_lobes_f64(3.0)
    x0 = planes_np[0].astype(np.float64)
    refs = [orc.fir_f64(x0, lob64[h], lob64[vv])[1] for h, vv in orc.GAUSS_OP_LOBES]
    for name, dt, es in (("f32", torch.float32, 4), ("f16", torch.float16, 2)):
        src = planes.to(dt)
        outs3 = [{k: torch.empty(planes.shape[1:], dtype=dt, device=dev) for k in range(6)} for _ in range(3)]

        def six():
            for k in range(3):
                g3.convolve_multi(src[k], outs3[k])
        r = rec(f"2b_gauss6_sigma3_3x1920x1080_{name}", six, planes.numel(), 7 * es * planes.numel())
        d_outs = [outs3[k][op] for k in range(3) for op in range(6)]
        r["e2e"] = _e2e(six, [_pinned(src)], [src], d_outs, [_pinned(t) for t in d_outs], planes.numel(), 10)
        six()
        torch.cuda.synchronize()
        errs = []
        for op in range(6):
            lh, lv = (lob[i] for i in orc.GAUSS_OP_LOBES[op])
            v = valid(x0.shape, len(lv) & ~1, len(lh) & ~1)
            errs.append(_err(F.FIRGaussianConvolver2.OPS[op], outs3[0][op].float().cpu().numpy()[v], refs[op][v]))
        r["errors_vs_fp64"] = errs
        r["errors_note"] = "plane 0; FP64 lobes and arithmetic on the u8 input"
    xs = [planes_np[k].astype(np.float32) for k in range(3)]
    r["cpu"] = {"gpix_per_s": _cpu_rate(lambda: [orc.fir_f32(x, lob[h], lob[vv]) for x in xs
                                                 for h, vv in orc.GAUSS_OP_LOBES], planes.numel(), max_reps=3),
                "threads": threads, "kind": "FP32 C restatement (oracle/), six operators"}
    res["2b_gauss6_sigma3_3x1920x1080_f32"]["cpu"] = r["cpu"]
    # next row: box sums of 4-channel float feature vectors (the SuperPixels
    # box filter), 15x15 windows, 3840x2160
    feat = torch.from_numpy(workloads.feature_image()).to(dev)
    fsum = torch.empty_like(feat)
    fbox = F.BoxFilter2(15, 15, 23)
    rec("next_features_box15_vec4_3840x2160_f32", lambda: fbox.convolve_vec(feat, fsum),
        feat.shape[0] * feat.shape[1], 2 * feat.numel() * 4)
    # next row: stereo cost aggregation, 7x7 windows, 64 disparities,
    # diff<u8>(50), disparity-major int32 costs of two 1920x1080 u8 images
    sl, sr = (torch.from_numpy(a).to(dev) for a in workloads.stereo_pair())
    scosts = torch.empty((64,) + tuple(sl.shape), dtype=torch.int32, device=dev)
    sbox = F.BoxFilter2(7, 7, 23)
    rec("next_stereo_w7_d64_1920x1080_u8_i32", lambda: sbox.convolve_stereo(sl, sr, scosts, 50),
        sl.numel() * 64, 2 * sl.numel() + 4 * 64 * sl.numel())
    res["next_stereo_w7_d64_1920x1080_u8_i32"]["unit"] = "G cost values/s (pixels x disparities)"
    # the step after it (DisparitySelector): winner-take-all disparities of the
    # valid cost region with the left-right check, into an int32 image
    sel = F.DisparitySelector(80, 2)
    disp = torch.zeros(sl.shape, dtype=torch.int32, device=dev)
    srows, scols = sl.shape[0] - 6, sl.shape[1] - 6
    rec("next_select_disparity_d64_1920x1080_i32", lambda: sel.select(scosts, disp, srows, scols, 3, 3),
        srows * scols, 4 * 64 * srows * scols + 4 * srows * scols)
    res["next_select_disparity_d64_1920x1080_i32"]["consistent_frac"] = round(
        float((disp[3:3 + srows, 3:3 + scols] == 80 - 9).float().mean()), 3)
    # next row: NPP's 15x15 Gaussian (the reference's nppGauss timing program)
    # beside this library's Gaussian of sigma 2 (17x17 support) on the same u8
    # image sizes; timing only, the coefficient sets differ
    exe = os.path.join(ROOT, "tucuda_gb300", "lib", "tucu_npp_gauss_time")
    for rows, cols, reps in ((1080, 1920, 200), (6480, 11520, 20)):
        name = f"next_npp_gauss15x15_vs_smooth_sigma2_{cols}x{rows}_u8"
        h8 = ((np.arange(rows * cols, dtype=np.uint64) * np.uint64(2654435761)) >> np.uint64(11)) % np.uint64(256)
        x8 = torch.from_numpy(h8.astype(np.uint8).reshape(rows, cols)).to(dev)
        y8 = torch.empty_like(x8)
        fn = lambda: g2.smooth(x8, y8)
        fn()
        ms = time_events(fn, reps)
        entry = {"ours_gpix_per_s": round(rows * cols / (ms * 1e-3) / 1e9, 2), "ours_ms": round(ms, 4)}
        try:
            r = subprocess.run([exe, str(rows), str(cols), str(reps)], capture_output=True,
                               text=True, timeout=120)
            npp = json.loads(r.stdout.strip().splitlines()[-1]) if r.returncode == 0 else None
            entry["npp_gpix_per_s"] = npp["gpix_per_s"] if npp else None
            entry["npp_ms"] = npp["ms"] if npp else None
            if not npp:
                entry["npp_unavailable"] = (r.stderr or r.stdout).strip()[-200:]
        except (OSError, ValueError, subprocess.TimeoutExpired) as e:
            entry["npp_unavailable"] = str(e)[:200]
        res[name] = entry
    # 3: guided filter radius 8, eps = 0.01*255^2, 1920x1080 float32 and
    # reduced storage (input, guide and output in bf16 / f16)
    p_np, g_np = workloads.guided_pair()
    _, ref = orc.guided_f64(p_np.astype(np.float64), g_np.astype(np.float64), 17, 17, workloads.GUIDED_E)
    v = valid(p_np.shape, 16, 16)
    gf = F.GuidedFilter2(17, 17, workloads.GUIDED_E, 23)
    errs = []
    for name, dt, es in (("f32", torch.float32, 4), ("bf16", torch.bfloat16, 2), ("f16", torch.float16, 2)):
        p, gd = (torch.from_numpy(a).to(dev).to(dt) for a in (p_np, g_np))
        go = torch.empty_like(p)
        key = "3_guided_r8_1920x1080_f32" if name == "f32" else f"3_guided_r8_1920x1080_{name}_storage"
        r = rec(key, lambda: gf.convolve(p, gd, go), p.numel(), 3 * es * p.numel())
        r["e2e"] = _e2e(lambda: gf.convolve(p, gd, go), [_pinned(p), _pinned(gd)], [p, gd], [go],
                        [_pinned(go)], p.numel(), 20)
        gf.convolve(p, gd, go)
        torch.cuda.synchronize()
        errs.append(_err(f"guided, {name} storage", go.float().cpu().numpy()[v], ref[v]))
    r3 = res["3_guided_r8_1920x1080_f32"]
    r3["errors_vs_fp64"] = errs
    r3["errors_note"] = "FP64 oracle over the f32 inputs: reduced storage includes the input rounding"
    r3["cpu"] = {"gpix_per_s": _cpu_rate(lambda: orc.guided_f32(p_np, g_np, 17, 17, workloads.GUIDED_E),
                                         p_np.size),
                 "threads": threads, "kind": "FP32 C restatement (oracle/)"}
    return res


# ---- our arm ------------------------------------------------------------------------------

def nvtx_push(name):
    try:
        import torch
        torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def nvtx_pop():
    try:
        import torch
        torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def run_ours(args, rank, world, local):
    import torch
    from tucuda_gb300 import autotune
    from tucuda_gb300.batch import Batch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    jobs, ins, outs, inbuf, outbuf = build_workload(dev, "f16", rank, world)
    pixels = sum(j.pixels for j in jobs)
    from tucuda_gb300 import replicas
    total_pixels = replicas.sum_over_ranks(pixels) if world > 1 else pixels
    alg_bytes = sum(a.numel() * a.element_size() + b.numel() * b.element_size()
                    for a, b in zip(ins, outs))

    batch = Batch(tensor=True)
    add_jobs(batch, jobs, ins, outs)
    desc = {"workload": "batched", "jobs": [(j.op, j.rows, j.cols, j.sigma, j.radius) for j in jobs],
            "storage": "f16", "tensor": True}
    fr, br, table = autotune.tune(batch, desc, autotune.TENSOR_CANDIDATES)
    info = batch.info()

    if not args.only_batch:
        # the exact FP32-pipe batch (bit-equal to the oracle) on the same workload
        exact = Batch()
        add_jobs(exact, jobs, ins, outs)
        efr, ebr, _ = autotune.tune(exact, {**desc, "tensor": False})
        time_events(exact.launch, 3)
        exact_ms = time_events(exact.launch, 40)
        exact_info = exact.info()
        del exact
        # plain single-image FP32 path on the same workload (per-image launches)
        jobs32, ins32, outs32, in32, out32 = build_workload(dev, "f32", rank, world)
        plain_pass(jobs32, ins32, outs32)
        plain_ms = time_events(lambda: plain_pass(jobs32, ins32, outs32), 3)
        plain_fp16_ms = time_events(lambda: plain_pass(jobs, ins, outs), 3)
        tcache = ({}, {})
        plain_pass(jobs, ins, outs, True, tcache)
        plain_tc_ms = time_events(lambda: plain_pass(jobs, ins, outs, True, tcache), 3)
        del jobs32, ins32, outs32, in32, out32
        torch.cuda.empty_cache()

    # ---- timed region: K graph launches ----
    for _ in range(args.warmup):
        batch.launch()
    torch.cuda.synchronize()
    barrier(world)
    stream = torch.cuda.current_stream()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        nvtx_push("timed")  # profilers select the timed launches by this range
        s.record(stream)
        for _ in range(args.steps):
            batch.launch()
        e.record(stream)
        torch.cuda.synchronize()
        nvtx_pop()
    ms = s.elapsed_time(e) / args.steps
    barrier(world)
    ms_max = max_over_ranks(ms, world)
    value = total_pixels / (ms_max * 1e-3) / 1e9
    if args.only_batch:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 3), "unit": METRIC,
                              "ms_per_step": round(ms_max, 4), "kernels_per_launch": info["kernels"],
                              "only_batch": True}), flush=True)
        return

    # ---- end to end through the public API on host images (tucu_pipe_*):
    # pinned host -> device copies, the batch, device -> host copies of the
    # valid outputs, in groups whose copies overlap other groups' kernels ----
    from tucuda_gb300 import hostmem
    from tucuda_gb300.batch import HostBatch
    h_in = torch.empty(inbuf.shape, dtype=inbuf.dtype, pin_memory=True)
    h_in.copy_(inbuf)
    h_out = torch.empty(outbuf.shape, dtype=outbuf.dtype, pin_memory=True)

    def host_view(hbuf, dbuf, t):
        off = (t.data_ptr() - dbuf.data_ptr()) // t.element_size()
        rows, cols = t.shape
        return hbuf.view(-1)[off:off + t.stride(0) * rows].view(rows, t.stride(0))[:, :cols]

    # The host slabs mirror the device slabs, so each group moves as one byte
    # range per direction (span copies).
    hb = HostBatch(chunks=E2E_CHUNKS, spans=True, tensor=True)
    for j, a, b in zip(jobs, ins, outs):
        ha, hbo = host_view(h_in, inbuf, a), host_view(h_out, outbuf, b)
        if j.op == "gauss":
            hb.add_gauss(ha, a, hbo, b, j.sigma)
        else:
            hb.add_box(ha, a, hbo, b, j.window, j.window, normalize=True)
    hb.plan(fr, br)
    hinfo = hb.info()
    hb.run()
    torch.cuda.synchronize()
    barrier(world)
    e2e_ms = max_over_ranks(time_events(hb.run, max(3, min(args.steps, 20))), world)
    e2e_value = total_pixels / (e2e_ms * 1e-3) / 1e9
    host_numa = hostmem.numa_report({"inputs": h_in, "outputs": h_out}, local)

    # Serving traces at the low, middle and high arrival rates of the
    # configuration (SERVING_RUNS).
    serving = [run_serving(n=n, rate=r) for r, n in SERVING_RUNS] if rank == 0 else None
    configs = run_configs(dev, peaks()[0]) if rank == 0 else None
    peak, peak_kind = peaks()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    traffic = profiled_traffic()
    clk = clocks.summary()

    if rank != 0:
        return
    # About 10 s of CPU work: passes over a ~256 Mpix sample of the workload.
    sample, cpx = cpu_prepare(CPU_SAMPLE_MPIX)
    cdesc, cpu_threads = cpu_desc(sample, cpx)
    cpu_time(sample[:1])
    spent, passes = 0.0, 0
    while passes < 1 or (spent < 10.0 and passes < 8):
        spent += cpu_time(sample)
        passes += 1
    cpu_v = passes * cpx / spent / 1e9
    cdesc += f", {passes} passes"
    batch.launch()  # the outputs the report reads come from the timed (tensor-core) path
    torch.cuda.synchronize()
    precision = precision_report(jobs, ins, outs)
    if configs is not None:
        configs["next_extrema_min15_3x1920x1080_u8_val_pos"]["cpu"] = cpu_extrema()
        configs["next_stereo_w7_d64_1920x1080_u8_i32"]["cpu"] = cpu_stereo()
        configs["next_select_disparity_d64_1920x1080_i32"]["cpu"] = cpu_select()
        configs["next_features_box15_vec4_3840x2160_f32"]["cpu"] = cpu_features()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max, 4),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f16",
        "data": "synthetic (seeded uniform [0,255) pixels, FP16 storage)",
        "config": {"workload": WORKLOAD, "images": len(jobs), "mpix": round(pixels / 1e6, 1),
                   "storage": "f16", "accumulate": "f32", "arithmetic": ARITHMETIC,
                   "l2": "inputs 1.36 GB > 129 MB L2; no flush",
                   "tile_rows": {"fir": fr, "box": br}, "work_items": info["items"],
                   "kernels_per_launch": info["kernels"],
                   "parallelism": f"replicas x{world}" + (", the 256 images sharded across ranks" if world > 1 else "")},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_kind": peak_kind, "kernel": "fir_tc_kernel<__half> (every job of the batch)",
                     "algorithmic_bytes_per_launch": alg_bytes},
        "cpu_baseline": {"value": round(cpu_v, 4), "unit": METRIC, "cores": cpu_threads,
                         "kind": "port", "sample": cdesc},
        "e2e": {"value": round(e2e_value, 3), "unit": METRIC, "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": int(hinfo["h2d_bytes"]),
                "d2h_bytes_per_step": int(hinfo["d2h_bytes"]),
                "api": f"tucu_pipe_run (HostBatch), {hinfo['groups']} groups, pinned host slabs "
                       "mirroring the device slabs, one span copy per group and direction",
                "host_numa": host_numa},
        "gpu_launches": args.steps * info["kernels"],
        "clocks": clk,
        "exact_fp32_pipe": {"gpix_s": round(pixels / (exact_ms * 1e-3) / 1e9, 3),
                            "ms_per_step": round(exact_ms, 4), "tile_rows": {"fir": efr, "box": ebr},
                            "kernels_per_launch": exact_info["kernels"],
                            "note": "the FP32-pipe batch, bit-equal to the oracle"},
        "plain_fp32_gpix_s": round(pixels / (plain_ms * 1e-3) / 1e9, 3),
        "plain_fp16_gpix_s": round(pixels / (plain_fp16_ms * 1e-3) / 1e9, 3),
        "plain_fp16_tensor_gpix_s": round(pixels / (plain_tc_ms * 1e-3) / 1e9, 3),
        "batched_over_plain_fp32": round(plain_ms / ms, 3),
        "autotune_ms": table.get("ms"),
        "serving": serving,
        "configs_1_to_3": configs,
        "precision": precision,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--only-batch", action="store_true",
                    help="time the batched graph launches only (for profiling runs)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
