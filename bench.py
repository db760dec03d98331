"""Benchmark: tomograms/s of the hologram -> RI path on one GB300 (or N replicas).

Workloads (seeded synthetic data with the shapes of the benchmark configurations;
see ctdm_gb300.phantom):
  plain_small  49 x 256^2 holograms -> 256^3, DCT unwrap, 10 positivity iterations
  wrap_heavy   121 x 1024^2 holograms -> 256^2 windows -> 256^3, DCT + Goldstein, 20 iterations

`value`  tomograms/s with holograms resident in HBM (CUDA events per step, L2
         flushed between steps by writing a 256 MiB buffer outside the timed region).
`e2e`    the same through the C ABI with pinned host buffers as a stream of
         tomograms (ctdm_submit per step, one ctdm_wait; host clock): every step's
         H2D copy of the holograms and D2H copy of the RI volume are inside the timed
         region, with consecutive calls' copies and kernels overlapping.
         `one_call_at_a_time` is the same through ctdm_reconstruct, which waits for
         its volume before the next call.
`--impl reference` times the FP64 CPU implementation of the path on the host
cores (the reference's path is CUDA; its CPU restatement is the oracle).
`--config cufft` compares this library's transforms and loop with cuFFT on the same GPU.
`--config large` runs 16 tomograms at 768^3 through the batched scheduler with admission
by free device memory.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "plain_small": dict(iterations=10, goldstein=False),
    "wrap_heavy": dict(iterations=20, goldstein=True),
    "batched": dict(iterations=10, goldstein=False, tomograms=64, lanes=4),
    "gradient": dict(iterations=10, goldstein=False),
    "gradient_small": dict(iterations=10, goldstein=False),
    "pocs": dict(iterations=10, goldstein=False, angles=121, pocs_iterations=100, tv_steps=20),
    "cufft": dict(iterations=0, goldstein=False),
    "large": dict(iterations=40, goldstein=False, tomograms=16, angles=181, holo=2048, window=768, volume=768),
}


# Workloads measured on one GPU whatever the launch (the replicated N-GPU contract is the
# headline workloads'); under torchrun the other ranks exit at once.
SECONDARY = ("batched", "gradient", "gradient_small", "pocs", "cufft", "large")


def make_workload(name, seed):
    from ctdm_gb300 import phantom
    if name == "plain_small":
        return phantom.config_plain_small(seed=seed)
    if name == "wrap_heavy":
        return phantom.config_wrap_heavy(seed=seed)
    raise ValueError(name)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(values, device=None):
    """Per-rank timings -> their maximum over the ranks (the job takes as long as its
    slowest replica); the values unchanged without an initialised process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def whole_job_rate(world, units_per_rank, ms):
    """Units of all replicas (each rank processes units_per_rank) per second of the
    slowest rank's `ms`."""
    return world * units_per_rank / (ms / 1e3)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel, workload):
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of `kernel`
    at `workload` from the committed ncu summary profiles/traffic.md, whose table rows
    read `| workload | stage | bytes per launch | ... |`; None when it has no entry."""
    p = os.path.join(ROOT, "profiles", "traffic.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) >= 3 and cells[0] == workload and cells[1] == kernel:
            try:
                return float(cells[2])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------- CPU baseline (oracle)
def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    return O


def cpu_tomogram(O, acq, iters, goldstein):
    """One whole tomogram through the FP64 CPU implementation of the path (the oracle's
    or_tomogram: QPI, Goldstein when configured, DCT unwrap, resize, median, spectra in
    parallel over the angles on every host thread, then the Ewald mapping and the
    positivity loop).  Returns its wall time in seconds."""
    par = O.make_params(acq.n_holo, acq.m_crop, acq.r_vol, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    t0 = time.perf_counter()
    O.tomogram(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y, run_goldstein=goldstein)
    return time.perf_counter() - t0


def cpu_sample(acq, iters, goldstein=False, min_seconds=10.0, max_tomograms=3):
    """The CPU baseline beside the GPU number: whole tomograms of the same workload,
    measured (not extrapolated), until `min_seconds` have passed or `max_tomograms` ran.
    Returns (seconds per tomogram, threads, text)."""
    O = oracle_module()
    nthr = O.get_threads()
    times = []
    while len(times) < max_tomograms and sum(times) < min_seconds:
        times.append(cpu_tomogram(O, acq, iters, goldstein))
    per = sum(times) / len(times)
    text = (f"measured: {len(times)} whole tomogram(s) of this workload through the FP64 oracle "
            f"({len(acq.ang_x)} angles{' with Goldstein' if goldstein else ''}, {iters} iterations at "
            f"{acq.r_vol}^3) on {nthr} host threads, {per:.2f} s each")
    return per, nthr, text


def workload_config(name, acq, world):
    """The `config` object of both arms' lines for workload `name`."""
    cfg = CONFIGS[name]
    return {"workload": name, "holograms": f"{len(acq.ang_x)}x{acq.n_holo}^2", "window": acq.m_crop,
            "volume": f"{acq.r_vol}^3", "iterations": cfg["iterations"], "goldstein": cfg["goldstein"],
            "parallelism": f"replicas{world}", "l2": "flushed between steps (256 MiB write)"}


# ---------------------------------------------------------------- batched workload
def batched_jobs(dev, seed=3000, count=64, iterations=10):
    """`count` tomograms: angle counts uniform in [31, 181], holograms 512^2 or 1024^2,
    volumes 256^3 or 384^3 (seeded).  Two seeded random multi-ellipsoid cells (2-6
    ellipsoids, RI 1.35-1.40), one per hologram size, are acquired at 181 cone angles;
    a tomogram with A angles takes A of them spread evenly over the cone, gathered on
    the device."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    rng = np.random.default_rng(seed)
    bases = {}
    for n in (512, 1024):
        cell = phantom.random_cell(np.random.default_rng(seed + n), n * 0.1e-6)
        acq = phantom.acquisition(n, 256, 181, na=0.9, seed=seed + n, ells=cell)
        bases[n] = (acq, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev))
    jobs, meta = [], []
    for _ in range(count):
        a = int(rng.integers(31, 182))
        n = int(rng.choice([512, 1024]))
        r = int(rng.choice([256, 384]))
        acq, holo, bg = bases[n]
        idx = np.round(np.linspace(0, 180, a)).astype(np.int64)
        h = holo.index_select(0, torch.from_numpy(idx).to(dev)).contiguous()
        p = C.default_params(n_holo=n, m_crop=n // 4, r_vol=r, iterations=iterations, n_med=acq.n_med,
                             wavelength=acq.wavelength, dx=acq.dx)
        out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
        jobs.append((p, h, bg, acq.ang_x[idx], acq.ang_y[idx], out))
        meta.append((a, n, r))
    return jobs, meta


def run_batched(args):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import build
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    cfg = CONFIGS["batched"]
    jobs, meta = batched_jobs(dev, seed=3000 + rank, count=cfg["tomograms"], iterations=cfg["iterations"])
    stream = torch.cuda.current_stream(dev)
    ctx = C.Context(local)

    def one_by_one():
        for (p, h, bg, ax, ay, out) in jobs:
            ctx.reconstruct_device(p, h, bg, ax, ay, out, stream=stream)

    lanes = args.lanes if args.lanes > 0 else cfg["lanes"]
    batch = C.Batch(lanes=lanes, device=local)
    batch.plan(jobs)
    for _ in range(args.warmup):
        batch.run(stream)
        one_by_one()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)

    def timed(fn):
        total = 0.0
        for _ in range(args.steps):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            total += a.elapsed_time(b)
        return total

    launches0 = C.launch_count()
    ms_graph = timed(lambda: batch.run(stream))
    ms_single = timed(one_by_one)
    launches = C.launch_count() - launches0
    clocks = sampler.stop()
    tomos = len(jobs) * args.steps
    # where the one-by-one time goes: the latency-bound per-angle front end (the part other
    # lanes can hide) against the bandwidth-bound volume passes (which share HBM when lanes
    # overlap them, so they cannot gain from running side by side)
    ctx.set_timing(True)
    one_by_one()
    torch.cuda.synchronize()
    st = ctx.stage_times()
    ctx.set_timing(False)
    front = sum(st[k][0] for k in ("qpi", "unwrap", "goldstein", "spectra", "ewald"))
    volume = sum(st[k][0] for k in ("y_inverse", "x_pass", "y_forward", "z_pass", "x_final"))
    split = {"front_end_ms": front, "volume_passes_ms": volume, "front_end_fraction": front / (front + volume),
             "gain_bound_if_front_ends_hidden": (front + volume) / volume}
    line = {
        "metric": "tomograms/s (hologram->RI), batched",
        "value": tomos / (ms_graph / 1e3),
        "unit": "tomograms/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_graph / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32/c64",
        "data": "synthetic (two seeded random multi-ellipsoid cells acquired at 181 cone angles, Poisson noise)",
        "config": {"workload": "batched", "tomograms": len(jobs), "lanes": lanes,
                   "angles": [m[0] for m in meta], "holograms": [m[1] for m in meta],
                   "volumes": [m[2] for m in meta], "iterations": cfg["iterations"],
                   "parallelism": "one GPU (secondary workload)", "l2": "inputs and volumes far larger than L2"},
        "one_by_one": {"value": tomos / (ms_single / 1e3), "unit": "tomograms/s",
                       "ms_per_step": ms_single / args.steps},
        "speedup_vs_one_by_one": ms_single / ms_graph,
        "one_by_one_stage_split": split,
        "e2e": None,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line))
    batch.close()


# ---------------------------------------------------------------- large batched workload
def run_large(args):
    """16 tomograms of 181 x 2048^2 holograms with 768^2 windows, 768^3 complex64
    volumes, 40 iterations of the accelerated loop each (the projected gradient step
    with momentum, fused into the loop passes), through the batched scheduler with
    admission by free device memory: all 16 lanes are requested and the planner keeps
    the ones whose workspaces fit.  One seeded cell acquired at 181 cone angles is
    reconstructed 16 times (the sizes, not the values, set the cost).  Per-kernel GB/s
    come from one tomogram on a context with the stage timer (algorithmic bytes per
    launch / CUDA-event time)."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import build, phantom
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    cfg = CONFIGS["large"]
    n, m, r, A, T = cfg["holo"], cfg["window"], cfg["volume"], cfg["angles"], cfg["tomograms"]
    acq = phantom.acquisition(n, r, A, na=0.9, seed=5000 + rank, workers=16)
    acq.m_crop = m
    holo = torch.from_numpy(acq.holograms).to(dev)
    bg = torch.from_numpy(acq.background).to(dev)
    acq.holograms = None
    p = C.params_for(acq, cfg["iterations"], accelerated=1)
    peak, peak_kind = measured_peaks()
    # one tomogram with the stage timer: per-kernel times
    ctx = C.Context(local)
    one = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, one)
    torch.cuda.synchronize()
    ctx.set_timing(True)
    ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, one)
    torch.cuda.synchronize()
    stages = ctx.stage_times()
    ctx.set_timing(False)
    r3 = float(r) ** 3
    F2 = ctx.read_buffer(7, np.complex64)
    measured = int(np.count_nonzero((F2.real != 0) & (F2.imag != 0)))
    del F2
    scheme = C.loop_scheme(r, device=local)
    ztile = C.z_tile(r, device=local)
    per_launch_bytes = {"qpi": (A + 1) * (4.0 * n * n + 8.0 * m * m), "unwrap": A * 8.0 * m * m,
                        "spectra": A * (8.0 * m * m + 8.0 * r * r), "ewald": A * 8.0 * r * r + 16 * r3,
                        # the accelerated x pass also reads and writes the previous iterate
                        "x_pass": 16 * r3 + 16 * r3, "y_forward": 16 * r3, "y_inverse": 16 * r3,
                        # the z pass reads the measured samples packed per tile when its plan
                        # allows (z_tile > 0), else F2 whole
                        "z_pass": (16 * r3 + 8.0 * measured + 4 * r3 / ztile) if ztile else 24 * r3,
                        "x_final": 16 * r3}
    kernels = {}
    for k, (ms, cnt) in stages.items():
        if cnt and k in per_launch_bytes:
            avg = ms / cnt
            kernels[k] = {"launches": cnt, "ms_per_launch": round(avg, 4),
                          "gb_per_s": round(per_launch_bytes[k] / (avg * 1e-3) / 1e9, 1),
                          "frac_of_peak": round(per_launch_bytes[k] / (avg * 1e-3) / 1e9 / peak, 3)}
    t_one = sum(v[0] for v in stages.values())
    ctx.close()
    del ctx, one
    torch.cuda.empty_cache()
    # the batch: T tomograms, T lanes requested, admission decides
    jobs = [(p, holo, bg, acq.ang_x, acq.ang_y, torch.empty((r, r, r), dtype=torch.complex64, device=dev))
            for _ in range(T)]
    batch = C.Batch(lanes=T, device=local)
    free0 = torch.cuda.mem_get_info(dev)[0]
    batch.plan(jobs)
    lanes, per_lane, avail = batch.admission()
    stream = torch.cuda.current_stream(dev)
    warm, steps = max(1, min(args.warmup, 1)), max(1, min(args.steps, 3))
    for _ in range(warm):
        batch.run(stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = C.launch_count()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        batch.run(stream)
    b.record(stream)
    b.synchronize()
    launches = C.launch_count() - launches0
    clocks = sampler.stop()
    ms = a.elapsed_time(b) / steps
    line = {
        "metric": "tomograms/s (hologram->RI), large batched with admission by free HBM",
        "value": T / (ms / 1e3), "unit": "tomograms/s", "n_gpus": 1, "steps": steps, "warmup": warm,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/c64",
        "data": "synthetic (one seeded Rytov phantom at 181 cone angles, Poisson noise, reconstructed 16 times)",
        "config": {"workload": "large", "tomograms": T, "holograms": f"{A}x{n}^2", "window": m, "volume": f"{r}^3",
                   "iterations": cfg["iterations"], "method": "accelerated loop (projected gradient step with "
                   "momentum, fused)", "parallelism": "one GPU (secondary workload)",
                   "l2": "volumes of 3.6 GB (far larger than L2)"},
        "admission": {"lanes_requested": T, "lanes_admitted": lanes, "workspace_bound_per_lane_gb": per_lane / 1e9,
                      "available_gb": avail / 1e9, "free_before_plan_gb": free0 / 1e9},
        "one_tomogram": {"ms": t_one, "loop_scheme": scheme, "z_tile": ztile, "kernels": kernels, "peak_gbs": peak,
                         "peak_source": peak_kind},
        "ri_rmse_vs_fp64": "tests/test_gpu_large.py: 768^3 from 2048^2 holograms against the FP64 oracle",
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line))
    batch.close()


# ---------------------------------------------------------------- gradient form vs positivity loop
def run_gradient(args):
    """The differentiable form (FISTA on 1/2 ||P F V - y||^2 + lambda TV(V) with the
    hand-written adjoint, optionally with the positivity constraint as a proximal
    step) against the positivity loop on the same measured data:
    RI RMSE against the phantom's band-limited RI volume and device time, for a
    schedule of gradient iteration counts.  `value` is tomograms/s of the gradient
    form at the first iteration count whose RMSE is at most the loop's (front end
    included); null when none reaches it.  Beside it, the accelerated positivity loop
    (the projected gradient step at lambda 0 and unit step with momentum, fused into
    the loop passes) for 2..iterations steps through the whole path."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import build, phantom
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    cfg = CONFIGS[args.config]
    if args.config == "gradient":
        # 1024^2 holograms, 181 angles on a cone at NA 1.2, 512^3 volume
        acq = phantom.acquisition(1024, 512, 181, na=1.2, seed=4000 + rank)
    else:
        acq = phantom.config_plain_small(seed=1000 + rank)
    r = acq.r_vol
    iters = cfg["iterations"]
    ctx = C.Context(local)
    stream = torch.cuda.current_stream(dev)
    holo = torch.from_numpy(acq.holograms).to(dev)
    bg = torch.from_numpy(acq.background).to(dev)
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    p = C.params_for(acq, iters)
    p0 = C.params_for(acq, 0)
    for _ in range(args.warmup):
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)
    torch.cuda.synchronize()
    # plain method, whole path; and the path without loop bodies (front end + final pass)
    a, b = ev(), ev()
    a.record(stream)
    ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)
    b.record(stream)
    b.synchronize()
    t_plain = a.elapsed_time(b)
    n_plain = out.clone()
    a, b = ev(), ev()
    a.record(stream)
    ctx.reconstruct_device(p0, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)
    b.record(stream)
    b.synchronize()
    t_front = a.elapsed_time(b)
    ptr, nbytes = ctx.buffer(7)          # measured data F2 of that call
    truth_f2 = torch.from_numpy(phantom.f2_truth(acq)).to(dev)
    n_true = torch.empty_like(out)
    ctx.positivity(truth_f2, r, 0, acq.k2, acq.n_med, n_true)
    del truth_f2
    torch.cuda.synchronize()

    def rmse(x):
        return float(torch.sqrt(torch.mean(torch.abs(x - n_true) ** 2)))

    rmse_plain = rmse(n_plain)
    tape = C.Tape(ptr, r, acq.k2, device=local)
    V = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    n_g = torch.empty_like(out)
    runs = []
    best = None
    for pos, lam in ((True, 0.0), (True, 1e-4), (False, 0.0), (False, 1e-3)):
        for j in (2, 3, 4, 5, 6, 8, 10, 20, 40):
            V.zero_()
            torch.cuda.synchronize()
            a, b = ev(), ev()
            a.record(stream)
            tape.reconstruct(V, j, lam=lam, eps=1e-3, step=1.0 if lam == 0.0 else 0.0, stream=stream,
                             positivity=pos)
            C.contrast_to_ri(V, r, acq.n_med, n_g, clamp=True, stream=stream)
            b.record(stream)
            b.synchronize()
            t = a.elapsed_time(b)
            e = rmse(n_g)
            runs.append({"positivity": pos, "lambda": lam, "iterations": j, "ms": round(t, 3), "ri_rmse": e})
            if e <= rmse_plain and (best is None or t < best["ms"]):
                best = {"positivity": pos, "lambda": lam, "iterations": j, "ms": t, "ri_rmse": e}
    tape.close()
    # the same projected iteration with momentum fused into the loop passes (accelerated
    # positivity loop: FISTA at lambda 0 and unit step), whole path from the holograms
    accel, accel_best = [], None
    for j in range(2, iters + 1):
        pa = C.params_for(acq, j, accelerated=1)
        ctx.reconstruct_device(pa, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)   # warm
        a, b = ev(), ev()
        a.record(stream)
        ctx.reconstruct_device(pa, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)
        b.record(stream)
        b.synchronize()
        t, e = a.elapsed_time(b), rmse(out)
        accel.append({"iterations": j, "ms": round(t, 3), "ri_rmse": e})
        if e <= rmse_plain and (accel_best is None or t < accel_best["ms"]):
            accel_best = {"iterations": j, "ms": t, "ri_rmse": e}
    t_grad = None if best is None else t_front + best["ms"]
    line = {
        "metric": "tomograms/s (hologram->RI), gradient form at the positivity loop's RI RMSE",
        "value": None if t_grad is None else 1e3 / t_grad,
        "unit": "tomograms/s",
        "n_gpus": 1,
        "steps": 1,
        "warmup": args.warmup,
        "ms_per_step": t_grad,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32/c64",
        "data": "synthetic (seeded Rytov phantom, Poisson noise); RMSE against the phantom's band-limited RI",
        "config": {"workload": args.config, "holograms": f"{len(acq.ang_x)}x{acq.n_holo}^2", "volume": f"{r}^3",
                   "positivity_iterations": iters},
        "plain": {"ms": t_plain, "ri_rmse": rmse_plain, "tomograms_per_s": 1e3 / t_plain},
        "front_end_ms": t_front,
        "gradient_best": best,
        "gradient_runs": runs,
        "accelerated_loop_best": accel_best,
        "accelerated_loop_runs": accel,
        "accelerated_loop_tomograms_per_s": None if accel_best is None else 1e3 / accel_best["ms"],
    }
    print(json.dumps(line))


def run_pocs(args):
    """ASD-POCS with TV on the frequency-interpolation mapping (the reference's
    BatchReconPOCS, its mathematics fixed) against the positivity loop on the same
    holograms: a one-axis scan of 121 angles (NA 0.9) of 256^2 holograms -> 256^3.
    RI RMSE against the phantom's band-limited RI volume and device time for a
    schedule of outer iteration counts (20 TV steps each).  `value` is tomograms/s of
    POCS at the reference's schedule (100 iterations of 20 TV steps), front end
    included."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import build, phantom
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    cfg = CONFIGS["pocs"]
    acq = phantom.acquisition(256, 256, cfg["angles"], na=0.9, seed=5000 + rank, scan="line")
    r, A = acq.r_vol, len(acq.ang_x)
    iters = cfg["iterations"]
    ctx = C.Context(local)
    stream = torch.cuda.current_stream(dev)
    holo = torch.from_numpy(acq.holograms).to(dev)
    bg = torch.from_numpy(acq.background).to(dev)
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def timed(fn):
        a, b = ev(), ev()
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    p = C.params_for(acq, iters)
    p0 = C.params_for(acq, 0)
    for _ in range(args.warmup):
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)
    torch.cuda.synchronize()
    t_plain = timed(lambda: ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream))
    n_plain = out.clone()
    t_front = timed(lambda: ctx.reconstruct_device(p0, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream))
    m = acq.m_crop
    ph_ptr, _ = ctx.buffer(2)      # unwrapped phase of that call (A*M*M)
    am_ptr, _ = ctx.buffer(1)      # amplitude
    U = torch.empty((A, r, r), dtype=torch.complex64, device=dev)
    F2 = torch.empty((r, r, r), dtype=torch.complex64, device=dev)

    def mapping():   # the loop path's spectra, then the frequency-interpolation mapping
        ctx.prepare_spectra(ph_ptr, am_ptr, U, A, m, acq.n_holo, r, stream=stream)
        ctx.map_fi(U, acq.ang_x, acq.fm0, acq.df, acq.dx, F2, stream=stream)

    mapping()
    t_map = timed(mapping)
    truth_f2 = torch.from_numpy(phantom.f2_truth(acq)).to(dev)
    n_true = torch.empty_like(out)
    ctx.positivity(truth_f2, r, 0, acq.k2, acq.n_med, n_true)
    del truth_f2
    torch.cuda.synchronize()

    def rmse(x):
        return float(torch.sqrt(torch.mean(torch.abs(x - n_true) ** 2)))

    runs = []
    for j in (1, 2, 5, 10, 20, 50, cfg["pocs_iterations"]):
        pp = C.pocs_params(iterations=j, tv_steps=cfg["tv_steps"])
        ctx.pocs(F2, r, acq.k2, acq.n_med, out, params=pp, stream=stream)   # warm
        t = timed(lambda: ctx.pocs(F2, r, acq.k2, acq.n_med, out, params=pp, stream=stream))
        runs.append({"iterations": j, "tv_steps": cfg["tv_steps"], "ms": round(t, 3), "ri_rmse": rmse(out)})
    loop = []
    for j in (0, 10, 20, 50):
        pj = C.params_for(acq, j)
        t = timed(lambda: ctx.reconstruct_device(pj, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream))
        loop.append({"iterations": j, "ms": round(t, 3), "ri_rmse": rmse(out)})
    full = runs[-1]
    t_total = t_front + t_map + full["ms"]
    per_iter = (runs[-1]["ms"] - runs[-2]["ms"]) / (runs[-1]["iterations"] - runs[-2]["iterations"])
    line = {
        "metric": "tomograms/s (hologram->RI), ASD-POCS + TV at the reference's 100 x 20 schedule",
        "value": 1e3 / t_total,
        "unit": "tomograms/s",
        "n_gpus": 1,
        "steps": 1,
        "warmup": args.warmup,
        "ms_per_step": t_total,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32/c64",
        "data": "synthetic (seeded Rytov phantom, Poisson noise, one-axis scan); RMSE against the phantom's "
                "band-limited RI",
        "config": {"workload": "pocs", "holograms": f"{A}x{acq.n_holo}^2 (AngX scan)", "volume": f"{r}^3"},
        "front_end_ms": t_front,
        "mapping_ms": t_map,
        "pocs_ms_per_iteration": per_iter,
        "pocs_runs": runs,
        "positivity_loop_runs": loop,
        "plain": {"ms": t_plain, "ri_rmse": rmse(n_plain), "iterations": iters},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- cuFFT comparison
def run_cufft_compare(args):
    """This library's transforms and positivity loop beside the same work built on cuFFT
    (through torch.fft, which calls cuFFT; comparison only, never on the product path),
    same GPU, same run, same data.  Per volume side R: one unnormalised 3-D transform
    (ctdm_fft's x / y / z line passes against a cuFFT 3-D plan), and one positivity-loop
    iteration (IFFT3, est_n, modify, FFT3, replacement of the measured voxels): the fused
    plane / z passes against cuFFT with the point operators as elementwise kernels.  Also
    the batched 2-D transforms of the front end (the per-angle spectra at 256^2 and the
    QPI hologram transforms at 1024^2).  Achieved GB/s counts one read and one write of
    the array per transform (16 bytes per complex point)."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import build
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    peak, peak_kind = measured_peaks()
    ctx = C.Context(local)
    k2 = float((2 * np.pi * 1.337 / 532e-9) ** 2)
    n_med = 1.337
    reps = max(args.steps, 3)

    def timed(fn, n=reps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(n):
            fn()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / n

    def gbs(nbytes, ms):
        return nbytes / (ms * 1e-3) / 1e9

    def torch_loop_iteration(G, F2, keep):
        V = torch.fft.ifftn(G, dim=(0, 1, 2))
        c = 1.0 - V / k2
        n = n_med * torch.sqrt(c)                        # principal root
        n = torch.complex(torch.clamp(n.real, min=n_med), torch.clamp(n.imag, min=0.0))
        f = (n * n / (n_med * n_med) - 1.0) * (-k2)
        G2 = torch.fft.fftn(f, dim=(0, 1, 2))
        return torch.where(keep, F2, G2)

    rows = []
    for r in (256, 384, 512):
        rng = np.random.default_rng(r)
        n3 = r ** 3
        x = torch.from_numpy((rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r)))
                             .astype(np.complex64)).to(dev)
        y = torch.empty_like(x)
        t_ours = timed(lambda: C.fft(x, [r, r, r]))
        t_cufft = timed(lambda: torch.fft.fftn(x, dim=(0, 1, 2), out=y))
        # loop iteration: measured data on 5 % of the voxels, ~1e-2 contrast
        keep_np = rng.random((r, r, r)) < 0.05
        f2 = np.where(keep_np, (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r))) * 20e-2 * k2,
                      0).astype(np.complex64)
        del x, y
        F2 = torch.from_numpy(f2).to(dev)
        out = torch.empty_like(F2)
        keep = torch.from_numpy(keep_np).to(dev)
        ctx.positivity(F2, r, 2, k2, n_med, out)          # tune / allocate
        t2 = timed(lambda: ctx.positivity(F2, r, 2, k2, n_med, out))
        t12 = timed(lambda: ctx.positivity(F2, r, 12, k2, n_med, out))
        t_ours_iter = (t12 - t2) / 10
        G = F2.clone()
        t_torch_iter = timed(lambda: torch_loop_iteration(G, F2, keep))
        rows.append({"R": r,
                     "fft3d": {"ctdm_ms": t_ours, "cufft_ms": t_cufft,
                               "ctdm_gbs": gbs(16.0 * n3, t_ours), "cufft_gbs": gbs(16.0 * n3, t_cufft)},
                     "loop_iteration": {"ctdm_fused_ms": t_ours_iter, "cufft_elementwise_ms": t_torch_iter,
                                        "speedup": t_torch_iter / t_ours_iter,
                                        "loop_scheme": C.loop_scheme(r, device=local)}})
        del F2, out, keep, G
        torch.cuda.empty_cache()
    batched = []
    for count, n in ((121, 256), (49, 256), (16, 1024)):
        rng = np.random.default_rng(n + count)
        x = torch.from_numpy((rng.standard_normal((count, n, n)) + 1j * rng.standard_normal((count, n, n)))
                             .astype(np.complex64)).to(dev)
        y = torch.empty_like(x)
        t_ours = timed(lambda: C.fft(x, [n, n], batch=count))
        t_cufft = timed(lambda: torch.fft.fft2(x, out=y))
        batched.append({"batch": count, "side": n, "ctdm_ms": t_ours, "cufft_ms": t_cufft,
                        "ctdm_gbs": gbs(16.0 * count * n * n, t_ours),
                        "cufft_gbs": gbs(16.0 * count * n * n, t_cufft)})
        del x, y
    line = {
        "metric": "FFT and positivity-loop time, this library vs cuFFT on the same GPU",
        "value": None, "unit": "ms", "n_gpus": 1, "steps": reps, "warmup": 2, "higher_is_better": False,
        "dtype": "c64", "data": "synthetic (seeded random volumes; measured data on 5% of the voxels)",
        "config": {"workload": "cufft", "parallelism": "one GPU (comparison workload)",
                   "l2": "volumes of 128 MiB and more (256^3 up)"},
        "peak_gbs": peak, "peak_source": peak_kind, "volumes": rows, "batched_2d": batched,
        "cufft": "torch.fft (cuFFT) with torch elementwise kernels; comparison only",
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU arm
def run_ours(args):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import build

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    cfg = CONFIGS[args.config]
    acq = make_workload(args.config, seed=1000 + rank)
    A = len(acq.ang_x)
    if args.loop_scheme >= 0:
        C.set_loop_scheme(acq.r_vol, args.loop_scheme, device=local)
    p = C.params_for(acq, cfg["iterations"], run_goldstein=int(cfg["goldstein"]))
    ctx = C.Context(local)
    holo = torch.from_numpy(acq.holograms).to(dev)
    bg = torch.from_numpy(acq.background).to(dev)
    r = acq.r_vol
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, out, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    launches0 = C.launch_count()
    # stage boundaries are recorded with CUDA events on the launching stream over the
    # whole timed loop (the library sums them per stage)
    ctx.set_timing(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    barrier()
    launches = C.launch_count() - launches0
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    stages = ctx.stage_times()
    ctx.set_timing(False)
    # e2e: host buffers through the C ABI (pinned), copies inside the timed region.  The
    # holograms are photon counts; when every value is an integer below 65536 they go up
    # as 16-bit counts (exact; widened to float on the GPU), else as float32.
    exact16 = bool(np.all(acq.holograms == np.rint(acq.holograms)) and acq.holograms.max() < 65536
                   and np.all(acq.background == np.rint(acq.background)) and acq.background.max() < 65536
                   and acq.holograms.min() >= 0 and acq.background.min() >= 0)
    up = np.uint16 if exact16 else np.float32
    h_holo = torch.from_numpy(acq.holograms.astype(up)).pin_memory()
    h_bg = torch.from_numpy(acq.background.astype(up)).pin_memory()
    h_out = torch.empty((r, r, r), dtype=torch.complex64).pin_memory()
    lib = C.load()
    e2e_fn = lib.ctdm_reconstruct_u16 if exact16 else lib.ctdm_reconstruct
    ax, ay = np.ascontiguousarray(acq.ang_x, np.float32), np.ascontiguousarray(acq.ang_y, np.float32)

    def e2e_step():
        C.check(e2e_fn(ctx.handle, ctypes.byref(p), A, h_holo.data_ptr(), h_bg.data_ptr(), ax.ctypes.data,
                       ay.ctypes.data, h_out.data_ptr()), "ctdm_reconstruct")

    e2e_step()
    torch.cuda.synchronize()
    barrier()
    # one call at a time: each ctdm_reconstruct waits for its volume
    sync_ms = 0.0
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(torch.cuda.default_stream(dev))
        e2e_step()
        b.record(torch.cuda.default_stream(dev))
        b.synchronize()
        sync_ms += a.elapsed_time(b)
    barrier()
    # a stream of tomograms: every step's holograms go up and its volume comes back, with
    # the calls in flight together (ctdm_submit, one ctdm_wait at the end; host clock).
    # The 254 MB of holograms uploaded per step exceed L2, so no flush between steps.
    h_outs = [h_out, torch.empty((r, r, r), dtype=torch.complex64).pin_memory()]
    bpc = 2 if exact16 else 4
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        C.check(lib.ctdm_submit(ctx.handle, ctypes.byref(p), A, h_holo.data_ptr(), h_bg.data_ptr(), bpc,
                                ax.ctypes.data, ay.ctypes.data, h_outs[k % 2].data_ptr()), "ctdm_submit")
    C.check(lib.ctdm_wait(ctx.handle), "ctdm_wait")
    e2e_ms = (time.perf_counter() - t0) * 1e3
    barrier()
    clocks = sampler.stop()

    dev_ms, e2e_ms, sync_ms = reduce_max([dev_ms, e2e_ms, sync_ms], device=dev)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    r3 = float(r) ** 3
    # Algorithmic HBM bytes per launch of each timed stage.  With the plane scheme the
    # x-pass stage is the plane pass (whole planes' x and y transforms, 16 R^3 bytes);
    # the z pass reads the measured samples packed per tile (G in and out, the kept
    # values, one mask word per (tile of 16 lines, z)).
    scheme = C.loop_scheme(r, device=local)
    ztile = C.z_tile(r, device=local)
    F2 = ctx.read_buffer(7, np.complex64)
    measured = int(np.count_nonzero((F2.real != 0) & (F2.imag != 0)))
    del F2
    bytes_per = {"x_pass": 16 * r3, "y_forward": 16 * r3, "y_inverse": 16 * r3,
                 "z_pass": (16 * r3 + 8.0 * measured + 4 * r3 / ztile) if ztile else 24 * r3,
                 "ewald": A * 8.0 * r * r + 16 * r3}
    plane = {1: "plane_pass", 2: "plane_pass_4cta"}
    kernel_of = {"x_pass": plane.get(scheme, "x_pass"), "y_forward": "y_forward",
                 "y_inverse": "y_inverse", "z_pass": "z_pass_packed", "ewald": "ewald"}
    best = max(bytes_per, key=lambda k: stages[k][0])
    ms_total, cnt = stages[best]
    avg_ms = ms_total / max(cnt, 1)
    achieved = bytes_per[best] / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic(kernel_of[best], args.config)
    cpu_s, cores, text = cpu_sample(acq, cfg["iterations"], cfg["goldstein"])
    line = {
        "metric": "tomograms/s (hologram->RI)",
        "value": whole_job_rate(world, args.steps, dev_ms),
        "unit": "tomograms/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32/c64",
        "data": "synthetic (seeded Rytov phantom, Poisson noise)",
        "config": workload_config(args.config, acq, world),
        "e2e": {"value": whole_job_rate(world, args.steps, e2e_ms), "unit": "tomograms/s",
                "h2d_bytes_per_step": int(h_holo.numel() * h_holo.element_size() + h_bg.numel() * h_bg.element_size()),
                "upload": "uint16 counts (exact: integer photon counts)" if exact16 else "float32",
                "d2h_bytes_per_step": int(r3 * 8),
                "mode": "stream of tomograms: ctdm_submit per step, one ctdm_wait (host clock)",
                "one_call_at_a_time": whole_job_rate(world, args.steps, sync_ms)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": kernel_of[best], "stage": best, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "loop_scheme": scheme, "measured_voxels": measured,
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "bytes_per_launch": bytes_per[best], "avg_launch_ms": avg_ms},
        "stages_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in stages.items()},
        "clocks": clocks,
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "tomograms/s", "cores": cores, "kind": "port",
                         "sample": text},
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    """The reference arm: the path's CPU implementation (the FP64 oracle, a restatement
    of the reference's kernels; the reference itself is CUDA) on all host threads, one
    whole tomogram of the same workload per step, measured."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    if args.config == "pocs":
        print(json.dumps({"impl": "reference", "unavailable": "the reference's BatchReconPOCS is disabled in its "
                          "driver and does not compute a usable reconstruction as written"}))
        return
    if args.config in ("batched", "cufft", "large") or args.config.startswith("gradient"):
        print(json.dumps({"impl": "reference", "unavailable": f"the {args.config} workload has no reference "
                          "counterpart (the reference has one positivity-loop reconstruction per BatchRecon call)"}))
        return
    cfg = CONFIGS[args.config]
    acq = make_workload(args.config, seed=1000)
    O = oracle_module()
    cores = O.get_threads()
    for _ in range(args.warmup):
        cpu_tomogram(O, acq, cfg["iterations"], cfg["goldstein"])
    times = [cpu_tomogram(O, acq, cfg["iterations"], cfg["goldstein"]) for _ in range(args.steps)]
    total = sum(times)
    value = args.steps / total
    text = (f"measured: {args.steps} whole tomograms ({len(acq.ang_x)} angles"
            f"{' with Goldstein' if cfg['goldstein'] else ''}, {cfg['iterations']} iterations at {acq.r_vol}^3) "
            f"through the FP64 oracle on {cores} host threads, {total / args.steps:.2f} s each")
    line = {
        "impl": "reference",
        "metric": "tomograms/s (hologram->RI)",
        "value": value,
        "unit": "tomograms/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Rytov phantom, Poisson noise)",
        "config": workload_config(args.config, acq, world),
        "cpu_baseline": {"value": value, "unit": "tomograms/s", "cores": cores, "kind": "port", "sample": text},
        "e2e": {"value": value, "unit": "tomograms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="wrap_heavy", choices=sorted(CONFIGS))
    ap.add_argument("--lanes", type=int, default=0, help="batched workload: concurrent lanes (0: the default 4)")
    ap.add_argument("--loop-scheme", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="positivity-loop scheme of the volume side, with plan variants 0 for its passes "
                         "(-1: the autotuner's choice; profiles pin 2, the choice without a profiler)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, _ = dist_info()
    if args.impl == "ours" and args.config in SECONDARY and world > 1 and rank != 0:
        return   # secondary workloads measure one GPU: rank 0 alone runs and prints
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "batched":
        run_batched(args)
    elif args.config.startswith("gradient"):
        run_gradient(args)
    elif args.config == "pocs":
        run_pocs(args)
    elif args.config == "cufft":
        run_cufft_compare(args)
    elif args.config == "large":
        run_large(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
