"""Benchmark of the NUDIM dual-space reconstruction loop on GB300.

Metric: voxel-iterations per second = nz * np^2 * (outer HIO/ER iterations)
/ wall time of the iteration loop (one "step" = one outer iteration of the
whole volume: Z-FFT, 12 NFFT + 11 adjoint NFFT per Z-plane inside the
constraint + 10-step CGNR, inverse Z-FFT, denoise, HIO/ER).

Workload (default): the precision-form configuration, a 256^3 blob + shell
phantom simulated to 61 tilts (-60..60 deg step 2) of 384 x 256 pixels at
SNR 0.5, reconstructed at np = nx = 384, nz = 256, padangle 1, 50 HIO + 50
ER, anisotropic-diffusion denoise.  `value` is the mixed form (FP32
spreading/FFT/stencils, FP64 tables), inputs resident in HBM; `e2e` is the
same metric through the C ABI with host buffers (tilt series in, volume out,
setup included); `fp64_plain` is the FP64 form on the same job.  Further
legs on the same line: `batched` (48 uneven TV jobs stepped together, one
stream each), `serving` (Poisson arrivals into the continuous-batching
server, p50/p99 latency), `cpu_baseline` (the oracle port on the host cores,
a bounded sample), and with --large the 768^2 x 256 TV configuration with
its FP64 correction.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
       [--large] [--batch-jobs J] [--serve-jobs J] [--autotune]
       python bench.py --tv NZxNYxNX      (the TV kernels alone)
Under torchrun each rank runs an independent replica on its own GPU
(the path has no cross-rank exchange): value = all ranks' voxel-iterations
/ max rank time.
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
sys.path.insert(0, ROOT)

PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
CFG = "cfg2"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


# ------------------------------------------------------------------ ranks
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def log(msg):
    """Progress of the legs on stderr (stdout carries only the JSON line)."""
    print("[bench] " + msg, file=sys.stderr, flush=True)


def max_over_ranks(dist, v, device=None):
    """Largest value over ranks (the slowest rank's time)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v, device=None):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
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
        self.th.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workload
NZ_OVERRIDE = None  # --nz: fewer Z-planes, for small-case profiling only


def workload_config():
    import copy

    from nudim_gb300.synth import CONFIGS
    c = copy.deepcopy(CONFIGS[CFG])
    if NZ_OVERRIDE:
        c["phantom"]["shape"] = (NZ_OVERRIDE,) + tuple(c["phantom"]["shape"][1:])
        c["recon"]["nz"] = NZ_OVERRIDE
    return c, dict(c["recon"])


def job_kwargs(r, precision):
    import nudim_gb300 as ng
    return dict(nx=r["nx"], nz=r["nz"], np=r["np"], gam_min=r["gam_min"], gam_max=r["gam_max"],
                interval=r["interval"], padangle=r["padangle"], nhio=r["nhio"], ner=r["ner"],
                denoise=r["denoise"], weight=r["weight"], precision=precision,
                variant=ng.VARIANT_SERIAL)


def stream_events(job):
    import torch
    st = torch.cuda.ExternalStream(job.stream)
    return st, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def timed_steps(ctx, job, steps, nvtx=None):
    """Device time (ms) of `steps` outer iterations on the job's stream.
    `nvtx` names a push/pop range around the launches (a filter for ncu)."""
    import torch
    st, e0, e1 = stream_events(job)
    torch.cuda.synchronize()
    if nvtx:
        torch.cuda.nvtx.range_push(nvtx)
    e0.record(st)
    for _ in range(steps):
        job.step(1)
    e1.record(st)
    if nvtx:
        torch.cuda.nvtx.range_pop()
    e1.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


# DRAM bytes per Z-plane of the adjoint NFFT's two kernels, from ncu captures of
# 32-plane launches on the same geometry (profiles/spread_colifft_cfg2_32planes.md,
# which lists both): dram__bytes_read.sum + dram__bytes_write.sum / 32.
MEASURED_ADJOINT_TRAFFIC_PER_PLANE = ((75.449856e6 + 71.426048e6)      # k_spread_colifft
                                      + (100.737792e6 + 36.037120e6)) / 32  # k_rowifft_crop


def roofline_from_profile(prof, peak_gbs, peak_kind, r, csize, steps):
    """Roofline of the dominant kernel pair, the adjoint NFFT (k_spread_colifft +
    k_rowifft_crop).  Its unit is one Z-plane's adjoint NFFT, whose algorithmic bytes
    are those of the unfused NFFT: c (P^2 + 4 n^2 + M) -- coefficients, the n x n
    oversampled grid written, transformed (read + write) and read back, and the node
    values.  achieved = units x that / the two kernels' measured time."""
    total = sum(v[0] for v in prof.values())
    shares = {k: round(v[0] / total, 4) for k, v in prof.items() if v[1] > 0}
    P, nz = r["np"], r["nz"]
    n = 2 * (1 << (P - 1).bit_length())
    M = 181 * P
    unit = csize * (P * P + 4 * n * n + M)
    ms_s, n_s, _ = prof["spread"]
    ms_c, n_c, _ = prof["crop"]
    # 11 adjoint NFFTs of every Z-plane per outer iteration (CGNR: one before
    # the loop, one per step)
    units = 11 * nz * steps
    planes_per_launch = units / max(1, n_s)
    secs = (ms_s + ms_c) / 1e3
    achieved = units * unit / secs / 1e9
    return "adjoint NFFT", {
        "bound": "hbm", "kernel": "adjoint NFFT (k_spread_colifft + k_rowifft_crop)",
        "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
        "frac": round(achieved / peak_gbs, 4),
        "traffic": round(MEASURED_ADJOINT_TRAFFIC_PER_PLANE * planes_per_launch),
        "algorithmic_bytes_per_launch": unit * planes_per_launch,
        "algorithmic_bytes_per_unit": unit, "units_per_launch": planes_per_launch,
        "avg_launch_ms": (ms_s + ms_c) / n_s, "peak_source": peak_kind}, shares


def cpu_baseline_sample(proj, r, iters=1, threads=None):
    """The oracle (CPU restatement, FP64) on a bounded sample of the same job:
    `threads` Z-planes run the per-plane NFFT+CGNR work (one plane per host
    thread), the volume phases (Z-FFTs, denoise, constraints) run on the
    full volume; the plane phase is extrapolated linearly to nz planes."""
    from oracle import orc
    orc.build()
    threads = threads or os.cpu_count() or 1
    kw = dict(nx=r["nx"], nz=r["nz"], np=r["np"], gam_min=r["gam_min"], gam_max=r["gam_max"],
              interval=r["interval"], padangle=r["padangle"], nhio=r["nhio"], ner=r["ner"],
              denoise=r["denoise"], weight=r["weight"], nthreads=threads,
              plane_limit=min(threads, r["nz"]))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.time()
    R = orc.Recon(proj, **kw)
    t_setup = time.time() - t0
    R.iterate(iters)
    tp, tv = R.times()
    R.close()
    nplanes = kw["plane_limit"]
    t_iter = (tp * r["nz"] / nplanes + tv) / iters
    V = r["nz"] * r["np"] ** 2
    return {"value": V / t_iter, "unit": "voxel-iters/s", "cores": threads, "kind": "port",
            "sample": "%d outer iteration(s) of the same job; per-plane NFFT+CGNR on %d of %d "
                      "Z-planes (one per thread) extrapolated linearly, volume phases on the "
                      "full volume; setup %.1f s untimed" % (iters, nplanes, r["nz"], t_setup),
            "s_per_iter": t_iter}


def serving_specs(n_jobs, seed, big_share=0.1, nhio=10, ner=10, weight=1):
    """Uneven jobs of the batched/serving configurations: nx from
    {96,128,160,192,256}, nz from 32..256 step 16, pad = round16(U(1.25,1.5)
    * nx), symmetric max tilt U{45..70}, step {1,2,3}; a `big_share` of the
    jobs is 384 x 384 x 192 (pad 480..576).  TV denoise."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_jobs):
        if rng.uniform() < big_share:
            nx, nz = 384, 192
        else:
            nx = int(rng.choice([96, 128, 160, 192, 256]))
            nz = int(rng.integers(2, 17)) * 16
        npad = int(round(rng.uniform(1.25, 1.5) * nx / 16.0)) * 16
        step = int(rng.choice([1, 2, 3]))
        gmax = int(rng.integers(45, 71))
        gmax -= gmax % step
        out.append(dict(nx=nx, nz=nz, np=npad, gam_min=-gmax, gam_max=gmax, interval=step,
                        padangle=1, nhio=nhio, ner=ner, denoise=1, weight=weight, seed=seed + k))
    return out


def uneven_inputs(ctx, specs):
    """Seeded blob phantoms and noisy (SNR 1) GPU-simulated tilt series for
    `specs`; returns [(tilt series, job arguments)]."""
    import nudim_gb300 as ng
    from nudim_gb300.synth import add_noise, blob_phantom
    inputs = []
    for sp in specs:
        s = dict(sp)
        sd = s.pop("seed")
        nx, nz = s["nx"], s["nz"]
        vol = blob_phantom((nz, nx, nx), nblobs=30, radius=0.35 * nx, sigma_range=(2, 8),
                           amp_range=(0.2, 1.0), seed=sd)
        proj = ng.project_2d1d(ctx, vol, nx, s["gam_min"], s["gam_max"], s["interval"])
        inputs.append((add_noise(proj, 1.0, sd + 1), s))
    return inputs


def batched_bench(ctx, n_jobs, steps, warmup, precision, seed=20261206):
    """The batched configuration: `n_jobs` independent uneven tomograms
    (ner=30 ER iterations with TV, no HIO), all resident, stepped together
    by nudim_step (each job's iteration is a graph replay on its own stream,
    so small jobs overlap).  Timed: `steps` iterations of every job, host
    clock between two device-wide synchronizations."""
    import torch

    import nudim_gb300 as ng
    specs = serving_specs(n_jobs, seed, big_share=0.0, nhio=0, ner=30, weight=0)
    inputs = uneven_inputs(ctx, specs)
    t0 = time.perf_counter()
    jobs = []
    for proj, s in inputs:
        jb = ng.Job(ctx, precision=precision, **s)
        jb.set_projections(proj)
        jobs.append(jb)
    t_setup = time.perf_counter() - t0
    vox = sum(s["nz"] * s["np"] ** 2 for _, s in inputs)
    ctx.step(jobs, warmup)
    torch.cuda.synchronize()
    n0 = ng.lib().nudim_launch_count()
    t0 = time.perf_counter()
    ctx.step(jobs, steps)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    launches = int(ng.lib().nudim_launch_count() - n0)
    shares = serial_ms = None
    if warmup + steps < 30:
        # one more iteration of every job, one job at a time (events around
        # short kernels of one stream would otherwise also time the other
        # streams' kernels), with per-kernel-class CUDA events: each class's
        # share of the summed kernel time
        ctx.profile(True)
        t0 = time.perf_counter()
        for jb in jobs:
            ctx.step([jb], 1)
            torch.cuda.synchronize()
        serial_ms = 1e3 * (time.perf_counter() - t0)
        prof = ctx.profile_read()
        ctx.profile(False)
        total = sum(v[0] for v in prof.values())
        shares = {k: round(v[0] / total, 4) for k, v in prof.items() if v[1] > 0}
    for jb in jobs:
        jb.close()
    out = {"value": vox * steps / t, "unit": "voxel-iters/s", "jobs": n_jobs,
           "voxels_total": int(vox), "steps": steps, "warmup": warmup,
           "ms_per_step": 1e3 * t / steps, "gpu_launches": launches,
           "setup_s": t_setup, "kernel_time_share": shares,
           "serial_profiled_ms_per_step": serial_ms,
           "timer": "host clock between device-wide synchronizations (one stream per job)",
           "sizes": "nx {96..256}, nz 32..256 step 16, pad 1.25-1.5 nx, tilt +-45..70 step "
                    "1/2/3, ner=30, TV"}
    log("batched: %d jobs, %.1f ms/step, %.3e voxel-iters/s" % (n_jobs, out["ms_per_step"],
                                                                  out["value"]))
    return out


def serving_bench(ctx, n_jobs, rate, precision, seed=20261205):
    """Poisson arrivals at `rate` jobs/s into the continuous-batching server;
    returns p50/p99 arrival-to-result latency and completed jobs/s."""
    import torch

    import nudim_gb300 as ng
    inputs = uneven_inputs(ctx, serving_specs(n_jobs, seed))
    arrivals = np.cumsum(np.random.default_rng(seed + 7).exponential(1.0 / rate, n_jobs))
    free, _ = torch.cuda.mem_get_info()
    srv = ng.Server(ctx, int(0.7 * free), max_active=16)
    t0 = time.perf_counter()
    tickets = []
    for (proj, s), ta in zip(inputs, arrivals):
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        tickets.append(srv.submit(proj, precision=precision, **s))
    for t in tickets:
        srv.wait(t, volume=False)
    st = srv.stats()
    srv.close()
    log("serving: %d jobs, p50 %.3f s, p99 %.3f s" % (n_jobs, st.get("p50_s", -1), st.get("p99_s", -1)))
    st.update(arrival_rate_jobs_per_s=rate, jobs=n_jobs,
              voxels_per_job_mean=float(np.mean([s["nz"] * s["np"] ** 2 for _, s in inputs])))
    return st


def large_bench(ctx, steps=10, warmup=3):
    """The large-volume configuration: 512 x 512 x 256 blob + shell phantom,
    121 tilts (-60..60 step 1) at SNR 0.3, reconstructed at np = nx = 768,
    nz = 256 with --weight and TV; the mixed form with an FP64 corrective
    iteration every 10 iterations.  Timed: `steps` iterations after `warmup`
    (with steps = 10, exactly one corrective iteration), CUDA events on the
    job's stream.  Accuracy: relative L2 against the FP64 plain form after
    1 and after warmup + steps iterations, with and without the correction."""
    import nudim_gb300 as ng
    from nudim_gb300.synth import CONFIGS, MASTER_SEED, make_inputs
    c = CONFIGS["cfg5"]
    r = dict(c["recon"])
    t0 = time.perf_counter()
    vol, proj = make_inputs(ctx, "cfg5", seed=MASTER_SEED)
    del vol
    t_inputs = time.perf_counter() - t0
    total = warmup + steps
    V = r["nz"] * r["np"] ** 2
    snaps = {}

    def run(precision, correct, timed):
        kw = job_kwargs(r, precision)
        kw["correct_every"] = correct
        t0 = time.perf_counter()
        job = ng.Job(ctx, **kw)
        job.set_projections(proj)
        t_setup = time.perf_counter() - t0
        job.step(1)
        v1 = job.volume()
        job.step(warmup - 1)
        ms = timed_steps(ctx, job, steps) if timed else None
        if not timed:
            job.step(steps)
        vN = job.volume()
        job.close()
        return v1, vN, ms, t_setup

    v1c, vNc, ms, t_setup = run(ng.MIXED, 10, True)
    log("large: %.1f ms/iteration (mixed, FP64 correction every 10)" % (ms / steps))
    v1m, vNm, ms_plain, _ = run(ng.MIXED, 0, True)
    v164, vN64, ms64, _ = run(ng.FP64, 0, True)
    rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out = {"value": V * steps / (ms / 1e3), "unit": "voxel-iters/s", "steps": steps,
           "warmup": warmup, "ms_per_step": ms / steps,
           "mixed_plain_ms_per_step": ms_plain / steps, "fp64_ms_per_step": ms64 / steps,
           "config": {"workload": "512x512x256 blob+shell phantom, 121 tilts -60..60 step 1, "
                                  "SNR 0.3, np=nx=768, nz=256, padangle 1, --weight, TV, "
                                  "FP64 correction every 10 iterations",
                      "voxels": V},
           "rel_l2_vs_fp64_after_1": {"corrected": rl(v1c, v164), "mixed": rl(v1m, v164)},
           "rel_l2_vs_fp64_after_%d" % total: {"corrected": rl(vNc, vN64),
                                               "mixed": rl(vNm, vN64)},
           "setup_s": t_setup, "inputs_s": t_inputs}
    log("large: %.3e voxel-iters/s, vs FP64 after %d: corrected %.2e, mixed %.2e"
        % (out["value"], total, out["rel_l2_vs_fp64_after_%d" % total]["corrected"],
           out["rel_l2_vs_fp64_after_%d" % total]["mixed"]))
    return out


# ------------------------------------------------------------------ arms
def run_reference(args):
    ws, rank, local = dist_env()
    dist = init_dist(ws, "gloo")
    if rank != 0:
        barrier(dist)
        return 0
    import nudim_gb300 as ng
    from nudim_gb300 import build as nb
    from nudim_gb300.synth import add_noise, blob_phantom
    from oracle import orc
    c, r = workload_config()
    # the tilt series is simulated by the oracle's own 2D1D restatement
    orc.build()
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    vol = blob_phantom(seed=20261203, **c["phantom"])
    s = c["sim"]
    proj = add_noise(orc.project_2d1d(vol, s["np"], s["gam_min"], s["gam_max"], s["interval"]),
                     s["snr"], 20261204)
    kw = dict(nx=r["nx"], nz=r["nz"], np=r["np"], gam_min=r["gam_min"], gam_max=r["gam_max"],
              interval=r["interval"], padangle=r["padangle"], nhio=r["nhio"], ner=r["ner"],
              denoise=r["denoise"], weight=r["weight"], nthreads=threads,
              plane_limit=min(threads, r["nz"]))
    R = orc.Recon(proj, **kw)
    R.iterate(args.warmup)
    tp0, tv0 = R.times()
    R.iterate(args.steps)
    tp1, tv1 = R.times()
    R.close()
    n = kw["plane_limit"]
    t_iter = ((tp1 - tp0) * r["nz"] / n + (tv1 - tv0)) / args.steps
    V = r["nz"] * r["np"] ** 2
    value = V / t_iter
    line = {
        "impl": "reference", "metric": "voxel-iters/s", "value": value, "unit": "voxel-iters/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_iter * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_block(r),
        "cpu_baseline": {"value": value, "unit": "voxel-iters/s", "cores": threads,
                         "kind": "port",
                         "sample": "each step: 1 outer iteration, per-plane NFFT+CGNR on %d of "
                                   "%d Z-planes (one per thread) extrapolated linearly, volume "
                                   "phases on the full volume" % (n, r["nz"])},
        "e2e": {"value": value, "unit": "voxel-iters/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    barrier(dist)
    return 0


def config_block(r):
    return {"workload": "precision-form job: 256^3 blob+shell phantom, 61 tilts -60..60 step 2, "
                        "np=nx=384, nz=%d, padangle 1, --weight, 50 HIO + 50 ER, anisotropic "
                        "diffusion" % r["nz"],
            "weight": bool(r["weight"]),
            "nx": r["nx"], "np": r["np"], "nz": r["nz"], "tilts": 61, "polar_lines": 181,
            "nfft_grid": 1024, "nhio": r["nhio"], "ner": r["ner"], "denoise": "DIFFUSION",
            "cgnr_steps": 10, "parallelism": "replicas",
            "l2": "inputs larger than L2: the Z-frequency volume alone is 302 MB (FP32 complex)"}


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = init_dist(ws, "nccl")
    dev = torch.device("cuda", local)
    import nudim_gb300 as ng
    from nudim_gb300 import build as nb
    from nudim_gb300.synth import MASTER_SEED, make_inputs
    nb.build()
    peaks, peak_kind = load_peaks()
    c, r = workload_config()
    V = r["nz"] * r["np"] ** 2
    ctx = ng.Context(local, ng.CTX_AUTOTUNE if args.autotune else 0)
    vol, proj = make_inputs(ctx, CFG, seed=MASTER_SEED + rank, cfg=c)

    # ---- mixed form, device resident (the headline `value`)
    job = ng.Job(ctx, **job_kwargs(r, ng.MIXED))
    job.set_projections(proj)
    job.step(1)
    vol_mixed_1 = job.volume()
    job.step(args.warmup - 1)
    ctx.sync()
    vol_mixed_w = job.volume()
    barrier(dist)
    clocks = ClockSampler(local)
    clocks.start()
    n0 = ng.lib().nudim_launch_count()
    ms = timed_steps(ctx, job, args.steps, "timed")  # graph replay of each iteration
    launches = int(ng.lib().nudim_launch_count() - n0)
    clk = clocks.stop()
    ms_max = max_over_ranks(dist, ms, dev)
    value = ws * V * args.steps / (ms_max / 1e3)
    log("mixed: %.2f ms/iteration, %.3e voxel-iters/s, %d launches" % (ms_max / args.steps, value, launches))
    # per-kernel CUDA events on the job stream over further iterations of the
    # same job (event timing runs the launches eagerly, without graph replay)
    prof_steps = min(2, r["nhio"] + r["ner"] - args.warmup - args.steps)
    if prof_steps > 0:
        ctx.profile(True)
        ms_prof = timed_steps(ctx, job, prof_steps, "profiled")
        prof = ctx.profile_read()
        ctx.profile(False)
        top, roof, shares = roofline_from_profile(prof, peaks.get("hbm_gbs", 6800.0), peak_kind,
                                                  r, 8, prof_steps)
        roof["profiled_ms_per_step"] = ms_prof / prof_steps
        log("profiled pass: top kernel %s, %.1f%% of measured HBM" % (top, 100 * roof["frac"]))
    else:
        roof, shares = None, None
    job.close()

    # ---- e2e through the C ABI: host tilt series in, host volume out
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        job = ng.Job(ctx, **job_kwargs(r, ng.MIXED))
        t1 = time.perf_counter()
        job.set_projections(proj)
        job.sync()
        t2 = time.perf_counter()
        job.step(args.steps)
        job.sync()
        t3 = time.perf_counter()
        out = job.volume()
        t_e2e = time.perf_counter() - t0
        phases = {"job_create_s": t1 - t0, "set_projections_s": t2 - t1,
                  "iterations_s": t3 - t2, "volume_to_host_s": t0 + t_e2e - t3}
        job.close()
        t_e2e = max_over_ranks(dist, t_e2e, dev)
        e2e = {"value": ws * V * args.steps / t_e2e, "unit": "voxel-iters/s",
               "h2d_bytes_per_step": int(proj.nbytes // args.steps),
               "d2h_bytes_per_step": int(out.nbytes // args.steps),
               "includes": "job setup (tilt-series NFFT, slice reorder, initial inverse NFFT)",
               "phases": phases}
        log("e2e: %.3e voxel-iters/s" % e2e["value"])

    # ---- FP64 plain form on the same job (fewer steps: it is the slow form)
    v64 = ms64 = err = err1 = None
    fp64_steps = max(1, args.fp64_steps)
    if not args.no_fp64:
        job = ng.Job(ctx, **job_kwargs(r, ng.FP64))
        job.set_projections(proj)
        job.step(1)
        vol64_1 = job.volume()
        job.step(args.warmup - 1)
        ctx.sync()
        vol64_w = job.volume()
        ms64 = timed_steps(ctx, job, fp64_steps)
        job.close()
        ms64 = max_over_ranks(dist, ms64, dev)
        v64 = ws * V * fp64_steps / (ms64 / 1e3)
        err = float(np.linalg.norm(vol_mixed_w - vol64_w) / np.linalg.norm(vol64_w))
        err1 = float(np.linalg.norm(vol_mixed_1 - vol64_1) / np.linalg.norm(vol64_1))
        log("fp64: %.2f ms/iteration, mixed vs fp64 rel L2 %.2e" % (ms64 / fp64_steps, err))

    line = {
        "metric": "voxel-iters/s", "value": value, "unit": "voxel-iters/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded blob+shell phantom, GPU 2D1D tilt-series simulation, "
                "Gaussian noise at SNR 0.5",
        "config": config_block(r),
        "form": "mixed (FP32 spreading/FFT/stencils, compensated gather, FP64 node/KB tables)",
        "autotune": bool(args.autotune),
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "kernel_time_share": shares,
        "clocks": clk,
    }
    if v64 is not None:
        line["fp64_plain"] = {"value": v64, "unit": "voxel-iters/s",
                              "ms_per_step": ms64 / fp64_steps, "steps": fp64_steps}
        line["mixed_over_fp64"] = value / v64
        line["rel_l2_mixed_vs_fp64_after_1_iteration"] = err1
        line["rel_l2_mixed_vs_fp64_after_warmup"] = err
    if args.large:
        line["large"] = large_bench(ctx)
    if args.batch_jobs > 0:
        line["batched"] = {"mixed": batched_bench(ctx, args.batch_jobs, args.steps, args.warmup,
                                                  ng.MIXED)}
    if args.serve_jobs > 0:
        line["serving"] = {"mixed": serving_bench(ctx, args.serve_jobs, args.serve_rate, ng.MIXED)}
        if args.serve_fp64:
            line["serving"]["fp64_plain"] = serving_bench(ctx, args.serve_jobs, args.serve_rate,
                                                          ng.FP64)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample(proj, r)
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    barrier(dist)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def tv_micro(args):
    """nudim_tv alone: a seeded N(0, 0.3^2) volume of the given shape, 40 inner
    iterations per call, `warmup` untimed calls then `steps` calls timed with
    CUDA events on the launching stream; FP32 form, then FP64 (one call)."""
    import torch

    import nudim_gb300 as ng
    from nudim_gb300 import build as nb
    nb.build()
    shape = tuple(int(v) for v in args.tv.lower().split("x"))
    ctx = ng.Context(0)
    out = {"metric": "TV inner iterations x voxels per second", "shape": list(shape)}
    V = int(np.prod(shape))
    for prec, name, steps in ((ng.MIXED, "fp32", args.steps), (ng.FP64, "fp64", 1)):
        dt = torch.float32 if prec == ng.MIXED else torch.float64
        g = torch.Generator().manual_seed(1)
        v = (torch.randn(shape, dtype=torch.float64, generator=g) * 0.3).to(dt).cuda()
        st = torch.cuda.current_stream()
        for _ in range(args.warmup if prec == ng.MIXED else 1):
            ng.tv(ctx, v.data_ptr(), shape, prec, 0.2, 40, stream=st.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            ng.tv(ctx, v.data_ptr(), shape, prec, 0.2, 40, stream=st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"ms_per_call": ms, "ms_per_inner_iteration": ms / 40,
                     "value": 40 * V / (ms / 1e3),
                     "bytes_per_inner_iteration": 5 * (4 if prec == ng.MIXED else 8) * V}
        log("tv %s %s: %.2f ms per 40 inner iterations" % (name, args.tv, ms))
    ctx.close()
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain-form leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--large", action="store_true",
                    help="also run the large-volume configuration (768^2 x 256, ~3 min)")
    ap.add_argument("--batch-jobs", type=int, default=48,
                    help="jobs in the batched measurement (0: skip)")
    ap.add_argument("--serve-jobs", type=int, default=16,
                    help="jobs in the serving measurement (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=0.5, help="Poisson arrivals, jobs/s")
    ap.add_argument("--serve-fp64", action="store_true", help="also serve the FP64 form")
    ap.add_argument("--nz", type=int, default=0,
                    help="override the number of Z-planes (small-case profiling only)")
    ap.add_argument("--autotune", action="store_true",
                    help="context with NUDIM_CTX_AUTOTUNE (plan candidates timed per geometry)")
    ap.add_argument("--tv", default="",
                    help="NZxNYxNX: only time nudim_tv (40 inner iterations) on a volume of "
                         "that shape in both forms (a kernel micro-benchmark)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global NZ_OVERRIDE
    NZ_OVERRIDE = args.nz or None
    if args.tv:
        return tv_micro(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
