"""Benchmark of the NUDIM dual-space reconstruction loop on GB300.

Metric: voxel-iterations per second = nz * np^2 * (outer HIO/ER iterations)
/ wall time of the iteration loop (one "step" = one outer iteration of the
whole volume: Z-FFT, per Z-plane the constraint's NFFT and the 10-step
CGNR -- in the FP64 form a trafo and an adjoint NFFT per step as in the
reference, in the mixed form one adjoint NFFT and 11 passes of the normal
operator by Toeplitz embedding -- inverse Z-FFT, denoise, HIO/ER).

Workload (default): the precision-form configuration, a 256^3 blob + shell
phantom simulated to 61 tilts (-60..60 deg step 2) of 384 x 256 pixels at
SNR 0.5, reconstructed at np = nx = 384, nz = 256, padangle 1, 50 HIO + 50
ER, anisotropic-diffusion denoise.  `value` is the mixed form (FP32
spreading/FFT/stencils, FP64 tables), inputs resident in HBM; `e2e` is the
same metric through the C ABI with host buffers (tilt series in, volume out,
setup included); `fp64_plain` is the FP64 form on the same job (with its own
e2e and its roofline against the GPU's measured FP64 FMA rate).  Further
legs on the same line: `accuracy` (the whole 50 HIO + 50 ER at 16 Z-planes in
every form against the FP64 form, with the FP64 loop's own floors under
1e-15, 1e-13 and FP32-sized input perturbations), `small_config` (the
128^3, 20 ER, TV configuration: GPU time in both forms and the oracle on the
host cores), `batched` (48 uneven TV jobs stepped together, one stream
each), `serving` (Poisson arrivals into the continuous-batching server,
p50/p99 latency), `cpu_baseline` (the oracle on the host cores: whole
iterations of the workload's geometry at one Z-plane per thread, and on one
core), `large` (the 768^2 x 256 TV configuration's mixed form; with
--large also its FP64 form, FP64 correction and accuracy).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
       [--large] [--batch-jobs J] [--serve-jobs J] [--serve-rate R] [--serve-fp64
       [--serve-fp64-jobs J] [--serve-fp64-rate R]] [--no-accuracy] [--no-cfg1]
       [--autotune]
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


# DRAM bytes per Z-plane of the adjoint NFFT's three kernels, from ncu captures
# of 32-plane launches on the same geometry: dram__bytes_read.sum +
# dram__bytes_write.sum / 32.
MEASURED_ADJOINT_TRAFFIC_PER_PLANE = ((172.924160e6 + 216.713216e6)    # k_spread_gather
                                      + (268.486656e6 + 75.897088e6)   # k_colifft_fs
                                      + (100.737792e6 + 36.037120e6)) / 32  # k_rowifft_crop
# The same for the Toeplitz operator pass (k_rowfft_fs + k_col_toeplitz +
# k_rowifft_crop_fs in its p^H q mode) per circulant size, 32-plane launches:
# the row spectra between the passes stay partly in the 129 MB L2 at that size.
MEASURED_TOEPLITZ_TRAFFIC_PER_PLANE = {
    768: ((37.8e6 + 15.6e6)                 # k_rowfft_fs<.., 24, 32>
          + (80.3e6 + 17.5e6)               # k_col_toeplitz<.., 24, 32>
          + (113.3e6 + 13.4e6)) / 32,       # k_rowifft_crop_fs<.., 24, 32>
    1024: ((37.8e6 + 36.6e6)                # k_rowfft_fs
           + (109.1e6 + 42.6e6)             # k_col_toeplitz
           + (138.5e6 + 15.6e6)) / 32,      # k_rowifft_crop_fs
}


def roofline_from_profile(prof, peak_gbs, peak_kind, r, csize, steps):
    """Roofline of the dominant kernel group of the mixed form's iteration.

    - The Toeplitz operator pass of the CGNR (k_rowfft_fs + k_col_toeplitz +
      k_rowifft_crop_fs, class "toeplitz"): 11 per Z-plane and outer
      iteration (one before the loop, one per step).  Unit: one Z-plane's
      pass, c (3 P^2 + 4 P nt) bytes -- p in, T p out and p read again for
      p^H T p, and the P x nt row spectra written, read and written by the
      column pass, and read back (nt: the circulant's size, 768 for P = 384).
    - The adjoint NFFT (k_spread_gather + k_spread_fixup + k_colifft_fs +
      k_rowifft_crop_fs, classes "spread" + "crop"): 11 per Z-plane and outer
      iteration with the NFFT form of the CGNR, 1 with the Toeplitz form.
      Unit: c (P^2 + 4 n^2 + M) -- coefficients, the n x n oversampled grid
      written, transformed (read + write) and read back, and the node values.
    achieved = units x unit bytes / the group's measured time."""
    total = sum(v[0] for v in prof.values())
    shares = {k: round(v[0] / total, 4) for k, v in prof.items() if v[1] > 0}
    P, nz = r["np"], r["nz"]
    n = 2 * (1 << (P - 1).bit_length())
    M = 181 * P
    toep = prof.get("toeplitz", (0.0, 0, 0.0))
    groups = []
    if toep[1] > 0:
        units = 11 * nz * steps
        launches = toep[1] / 3.0  # three passes per launch of the group
        # the circulant: 768 points when 2P - 1 <= 768 < n, else n
        nt = 768 if (2 * P - 1 <= 768 < n and os.environ.get("NUDIM_TOEPLITZ_GRID") != "nfft") else n
        unit = csize * (3 * P * P + 4 * P * nt)
        tr = MEASURED_TOEPLITZ_TRAFFIC_PER_PLANE.get(nt)
        groups.append(("Toeplitz operator pass",
                       "Toeplitz operator pass (k_rowfft_fs + k_col_toeplitz + k_rowifft_crop_fs)",
                       toep[0], units, launches, unit, tr))
    ms_s, n_s, _ = prof["spread"]
    ms_c, n_c, _ = prof["crop"]
    units = (1 if toep[1] > 0 else 11) * nz * steps
    groups.append(("adjoint NFFT",
                   "adjoint NFFT (k_spread_gather + k_spread_fixup + k_colifft_fs + "
                   "k_rowifft_crop_fs)", ms_s + ms_c, units, max(1, n_c),
                   csize * (P * P + 4 * n * n + M), MEASURED_ADJOINT_TRAFFIC_PER_PLANE))
    top, kernel, ms, units, launches, unit, tr = max(groups, key=lambda g: g[2])
    planes_per_launch = units / launches
    achieved = units * unit / (ms / 1e3) / 1e9
    return top, {
        "bound": "hbm", "kernel": kernel,
        "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
        "frac": round(achieved / peak_gbs, 4),
        "traffic": round(tr * planes_per_launch) if tr else None,
        "algorithmic_bytes_per_launch": unit * planes_per_launch,
        "algorithmic_bytes_per_unit": unit, "units_per_launch": planes_per_launch,
        "avg_launch_ms": ms / launches, "peak_source": peak_kind,
        "groups_ms": {g[0]: round(g[2], 3) for g in groups}}, shares


def cpu_sample_inputs(r, nz):
    """The tilt series of the workload's geometry with `nz` Z-planes (the
    phantom cut to nz planes), simulated and noised by the oracle's own 2D1D
    restatement on the host."""
    import copy

    from nudim_gb300.synth import CONFIGS, add_noise, blob_phantom
    from oracle import orc
    c = copy.deepcopy(CONFIGS[CFG])
    c["phantom"]["shape"] = (nz,) + tuple(c["phantom"]["shape"][1:])
    vol = blob_phantom(seed=20261203, **c["phantom"])
    s = c["sim"]
    return add_noise(orc.project_2d1d(vol, s["np"], s["gam_min"], s["gam_max"], s["interval"]),
                     s["snr"], 20261204)


def cpu_time_iterations(r, nz, threads, warmup, steps):
    """The oracle (the CPU restatement, FP64) on the workload's geometry with
    nz Z-planes: `warmup` untimed outer iterations, then `steps` timed ones,
    every phase of each on the whole nz-plane volume (nothing extrapolated).
    Returns (seconds per iteration, voxels per iteration)."""
    from oracle import orc
    orc.build()
    proj = cpu_sample_inputs(r, nz)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    kw = dict(nx=r["nx"], nz=nz, np=r["np"], gam_min=r["gam_min"], gam_max=r["gam_max"],
              interval=r["interval"], padangle=r["padangle"], nhio=r["nhio"], ner=r["ner"],
              denoise=r["denoise"], weight=r["weight"], nthreads=threads)
    R = orc.Recon(proj, **kw)
    R.iterate(warmup)
    t0 = time.perf_counter()
    R.iterate(steps)
    t = (time.perf_counter() - t0) / steps
    R.close()
    return t, nz * r["np"] ** 2


def cpu_baseline_sample(r, threads=None, steps=2):
    """cpu_baseline: the oracle on the host cores, whole outer iterations of
    the workload's geometry with one Z-plane per thread (all threads), and
    with two Z-planes on one core (the single-thread figure)."""
    threads = threads or os.cpu_count() or 1
    nz = max(2, threads + (threads & 1))
    t, vox = cpu_time_iterations(r, nz, threads, 1, steps)
    t1, vox1 = cpu_time_iterations(r, 2, 1, 0, 1)
    return {"value": vox / t, "unit": "voxel-iters/s", "cores": threads, "kind": "port",
            "sample": "%d outer iterations (after 1 untimed) of the workload's geometry (np=nx=%d, "
                      "61 tilts, the same options) with nz=%d Z-planes, one per thread, every phase "
                      "on the whole volume, nothing extrapolated" % (steps, r["np"], nz),
            "s_per_iter": t,
            "single_core": {"value": vox1 / t1, "unit": "voxel-iters/s", "cores": 1,
                            "sample": "1 outer iteration, nz=2 Z-planes, one thread",
                            "s_per_iter": t1}}


def serving_specs(n_jobs, seed, big_share=0.1, nhio=20, ner=30, weight=1):
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
    """Poisson arrivals at `rate` jobs/s into the continuous-batching server
    of jobs of the serving configuration (the batched size mix plus 10 % of
    384 x 384 x 192, each 20 HIO + 30 ER with TV); returns p50/p99
    arrival-to-result latency and completed jobs/s."""
    import torch

    import nudim_gb300 as ng
    inputs = uneven_inputs(ctx, serving_specs(n_jobs, seed, big_share=0.1, nhio=20, ner=30))
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
              voxels_per_job_mean=float(np.mean([s["nz"] * s["np"] ** 2 for _, s in inputs])),
              iterations_per_job="20 HIO + 30 ER, TV",
              big_jobs=int(sum(1 for _, s in inputs if s["nx"] == 384)))
    return st


def accuracy_leg(ctx, r, nz=16, snaps=(1, 2, 5, 10, 50, 75, 100)):
    """Accuracy of the reduced-precision forms against the FP64 form on the
    workload's geometry (384^2 planes, 61 tilts, the same options) with nz
    Z-planes, over the whole 50 HIO + 50 ER: relative L2 of the volume after
    each iteration in `snaps`, for the FP64 form on a tilt series perturbed by
    1e-15, 1e-13 and 6e-8 (FP32's unit roundoff) relative -- the floors: how
    far the FP64 loop itself moves under FP64- and FP32-sized input changes --
    the mixed form, the mixed form with its HIO iterations in FP64
    (correct_every = -1) and with an FP64 iteration every 10th
    (correct_every = 10)."""
    import copy

    import nudim_gb300 as ng
    from nudim_gb300.synth import CONFIGS, MASTER_SEED, make_inputs
    c = copy.deepcopy(CONFIGS[CFG])
    c["phantom"]["shape"] = (nz,) + tuple(c["phantom"]["shape"][1:])
    rr = dict(r, nz=nz)
    vol, proj = make_inputs(ctx, None, seed=MASTER_SEED, cfg=c)
    total = rr["nhio"] + rr["ner"]
    snaps = [s for s in snaps if s <= total]

    def run(p, precision, correct=0):
        kw = job_kwargs(rr, precision)
        kw["correct_every"] = correct
        job = ng.Job(ctx, **kw)
        job.set_projections(p)
        out, done = {}, 0
        for sn in snaps:
            job.step(sn - done)
            done = sn
            out[sn] = job.volume()
        fp64_its = job.corrections() if precision == ng.MIXED else total
        job.close()
        return out, fp64_its

    rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    t0 = time.perf_counter()
    ref, _ = run(proj, ng.FP64)
    def pert(eps):
        return proj * (1.0 + eps * np.random.default_rng(1).standard_normal(proj.shape))
    res = {"rel_l2_vs_fp64": {}, "fp64_iterations": {}}
    for name, p, prec, corr in (("fp64_perturbed_1e-15", pert(1e-15), ng.FP64, 0),
                                ("fp64_perturbed_1e-13", pert(1e-13), ng.FP64, 0),
                                ("fp64_perturbed_6e-8", pert(6e-8), ng.FP64, 0),
                                ("mixed", proj, ng.MIXED, 0),
                                ("mixed_fp64_hio", proj, ng.MIXED, -1),
                                ("mixed_correct_10", proj, ng.MIXED, 10)):
        v, n64 = run(p, prec, corr)
        res["rel_l2_vs_fp64"][name] = {str(k): rl(v[k], ref[k]) for k in snaps}
        res["fp64_iterations"][name] = n64
    res.update(config="workload geometry with nz=%d Z-planes: np=nx=%d, 61 tilts, %d HIO + %d ER, "
                      "the workload's denoise and weighting" % (nz, rr["np"], rr["nhio"], rr["ner"]),
               snapshots=snaps, seconds=time.perf_counter() - t0)
    log("accuracy (nz=%d) after %d: floor(1e-13) %.2e, floor(6e-8) %.2e, mixed %.2e, "
        "FP64 HIO %.2e" % (
        nz, total, res["rel_l2_vs_fp64"]["fp64_perturbed_1e-13"][str(total)],
        res["rel_l2_vs_fp64"]["fp64_perturbed_6e-8"][str(total)],
        res["rel_l2_vs_fp64"]["mixed"][str(total)],
        res["rel_l2_vs_fp64"]["mixed_fp64_hio"][str(total)]))
    return res


def cfg1_leg(ctx, steps=5, cpu=True):
    """The small plain-form configuration (128^3 blob phantom, 41 tilts
    -60..60 step 3, np = 128, padangle 1, --weight, 20 ER with TV): GPU time
    per outer iteration in both forms (CUDA events on the job's stream, after
    2 warm-up iterations), and the oracle on the host cores -- all threads
    on the whole volume, and one thread on 8 of its Z-planes (the per-plane
    work dominates) -- 1 outer iteration each after setup."""
    import copy

    import nudim_gb300 as ng
    from nudim_gb300.synth import CONFIGS, MASTER_SEED, add_noise, blob_phantom
    from oracle import orc
    c = CONFIGS["cfg1"]
    r = dict(c["recon"])
    orc.build()
    vol = blob_phantom(seed=MASTER_SEED, **c["phantom"])
    s = c["sim"]
    proj = add_noise(orc.project_2d1d(vol, s["np"], s["gam_min"], s["gam_max"], s["interval"]),
                     s["snr"], MASTER_SEED + 1)
    V = r["nz"] * r["np"] ** 2
    out = {"config": "128^3 blob phantom, 41 tilts -60..60 step 3, np=nx=128, nz=128, "
                     "padangle 1, --weight, 20 ER, TV", "voxels": V}
    for name, prec in (("fp64_plain", ng.FP64), ("mixed", ng.MIXED)):
        job = ng.Job(ctx, **job_kwargs(r, prec))
        job.set_projections(proj)
        job.step(2)
        ms = timed_steps(ctx, job, steps)
        job.close()
        out[name] = {"ms_per_step": ms / steps, "value": V * steps / (ms / 1e3),
                     "unit": "voxel-iters/s"}
    if cpu:
        threads = os.cpu_count() or 1
        os.environ["OMP_NUM_THREADS"] = str(threads)
        kw = dict(nx=r["nx"], nz=r["nz"], np=r["np"], gam_min=r["gam_min"],
                  gam_max=r["gam_max"], interval=r["interval"], padangle=r["padangle"],
                  nhio=r["nhio"], ner=r["ner"], denoise=r["denoise"], weight=r["weight"])
        R = orc.Recon(proj, nthreads=threads, **kw)
        t0 = time.perf_counter()
        R.iterate(1)
        t_all = time.perf_counter() - t0
        R.close()
        sub = copy.deepcopy(c)
        sub["phantom"]["shape"] = (8,) + tuple(sub["phantom"]["shape"][1:])
        vol8 = blob_phantom(seed=MASTER_SEED, **sub["phantom"])
        proj8 = orc.project_2d1d(vol8, s["np"], s["gam_min"], s["gam_max"], s["interval"])
        R = orc.Recon(add_noise(proj8, s["snr"], MASTER_SEED + 1), nthreads=1,
                      **dict(kw, nz=8))
        t0 = time.perf_counter()
        R.iterate(1)
        t_one = time.perf_counter() - t0
        R.close()
        out["cpu_oracle"] = {
            "all_cores": {"cores": threads, "s_per_iter": t_all, "value": V / t_all,
                          "unit": "voxel-iters/s", "sample": "1 outer iteration, whole volume"},
            "single_core": {"cores": 1, "s_per_iter_8_planes": t_one,
                            "value": 8 * r["np"] ** 2 / t_one, "unit": "voxel-iters/s",
                            "sample": "1 outer iteration of the geometry with 8 Z-planes"}}
    log("cfg1: FP64 %.1f ms, mixed %.1f ms per iteration" % (out["fp64_plain"]["ms_per_step"],
                                                            out["mixed"]["ms_per_step"]))
    return out


def fp64_peak():
    """The FP64 and FP32 FMA rates of this GPU (bin/fp64_peak: independent FMA
    chains, CUDA events), or None when the probe is missing."""
    exe = os.path.join(ROOT, "nudim_gb300", "bin", "fp64_peak")
    try:
        out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        return json.loads(out.stdout.strip().splitlines()[-1]) if out.returncode == 0 else None
    except (OSError, ValueError, IndexError, subprocess.TimeoutExpired):
        return None


def large_quick(ctx, steps=3, warmup=2):
    """The large-volume configuration's mixed form alone (512 x 512 x 256
    blob + shell phantom, 121 tilts, np = nx = 768, nz = 256, --weight, TV):
    `steps` iterations after `warmup`, CUDA events on the job's stream.  The
    default bench line carries it; --large adds the FP64 form, the FP64
    correction and the accuracy comparison."""
    import nudim_gb300 as ng
    from nudim_gb300.synth import CONFIGS, MASTER_SEED, make_inputs
    r = dict(CONFIGS["cfg5"]["recon"])
    vol, proj = make_inputs(ctx, "cfg5", seed=MASTER_SEED)
    del vol
    V = r["nz"] * r["np"] ** 2
    t0 = time.perf_counter()
    job = ng.Job(ctx, **job_kwargs(r, ng.MIXED))
    job.set_projections(proj)
    job.sync()
    t_setup = time.perf_counter() - t0
    job.step(warmup)
    ms = timed_steps(ctx, job, steps)
    job.close()
    out = {"value": V * steps / (ms / 1e3), "unit": "voxel-iters/s", "steps": steps,
           "warmup": warmup, "ms_per_step": ms / steps, "setup_s": t_setup,
           "config": {"workload": "512x512x256 blob+shell phantom, 121 tilts -60..60 step 1, "
                                  "SNR 0.3, np=nx=768, nz=256, padangle 1, --weight, TV, "
                                  "mixed form", "voxels": V}}
    log("large (mixed): %.1f ms/iteration, %.3e voxel-iters/s" % (ms / steps, out["value"]))
    return out


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
    """The reference arm: the oracle (the CPU restatement of the reference's
    loop, FP64) on all host cores.  A step is one whole outer iteration of the
    workload's geometry with one Z-plane per host thread (every phase on the
    whole volume, nothing extrapolated), so the run ends within minutes."""
    ws, rank, local = dist_env()
    dist = init_dist(ws, "gloo")
    if rank != 0:
        barrier(dist)
        return 0
    c, r = workload_config()
    threads = os.cpu_count() or 1
    nz = r["nz"] if NZ_OVERRIDE else max(2, threads + (threads & 1))
    t_iter, vox = cpu_time_iterations(r, nz, threads, args.warmup, args.steps)
    value = vox / t_iter
    line = {
        "impl": "reference", "metric": "voxel-iters/s", "value": value, "unit": "voxel-iters/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_iter * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_block(r),
        "cpu_baseline": {"value": value, "unit": "voxel-iters/s", "cores": threads,
                         "kind": "port",
                         "sample": "each step: 1 whole outer iteration of the workload's geometry "
                                   "(np=nx=%d, 61 tilts, the same options) with nz=%d Z-planes, one "
                                   "per thread, every phase on the whole volume" % (r["np"], nz)},
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

    # ---- FP64 plain form on the same job (fewer steps: it is the slow form),
    # device resident and end to end through the C ABI
    v64 = ms64 = err = err1 = e2e64 = None
    fp64_steps = max(1, args.fp64_steps)
    if not args.no_fp64:
        t0 = time.perf_counter()
        job = ng.Job(ctx, **job_kwargs(r, ng.FP64))
        job.set_projections(proj)
        job.sync()
        t_setup64 = time.perf_counter() - t0
        job.step(1)
        vol64_1 = job.volume()
        job.step(args.warmup - 1)
        ctx.sync()
        vol64_w = job.volume()
        ms64 = timed_steps(ctx, job, fp64_steps)
        t0 = time.perf_counter()
        out64 = job.volume()
        t_out64 = time.perf_counter() - t0
        job.close()
        ms64 = max_over_ranks(dist, ms64, dev)
        v64 = ws * V * fp64_steps / (ms64 / 1e3)
        # end to end: the same phases as the mixed form's e2e (setup, the
        # iterations, the volume to the host), the iterations timed above
        t_e2e64 = max_over_ranks(dist, t_setup64 + ms64 / 1e3 + t_out64, dev)
        e2e64 = {"value": ws * V * fp64_steps / t_e2e64, "unit": "voxel-iters/s",
                 "h2d_bytes_per_step": int(proj.nbytes // fp64_steps),
                 "d2h_bytes_per_step": int(out64.nbytes // fp64_steps),
                 "phases": {"job_create_and_set_projections_s": t_setup64,
                            "iterations_s": ms64 / 1e3, "volume_to_host_s": t_out64}}
        err = float(np.linalg.norm(vol_mixed_w - vol64_w) / np.linalg.norm(vol64_w))
        err1 = float(np.linalg.norm(vol_mixed_1 - vol64_1) / np.linalg.norm(vol64_1))
        log("fp64: %.2f ms/iteration, mixed vs fp64 rel L2 %.2e" % (ms64 / fp64_steps, err))
    peak64 = fp64_peak() if not args.no_fp64 else None
    acc = None
    if not args.no_accuracy:
        acc = accuracy_leg(ctx, r, nz=args.accuracy_nz)
    small = None
    if not args.no_cfg1:
        small = cfg1_leg(ctx, cpu=rank == 0 and not args.no_cpu)

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
        P, nz = r["np"], r["nz"]
        n = 2 * (1 << (P - 1).bit_length())
        M = 181 * P
        # FP64 flops of one outer iteration in the reference's parameters: per
        # Z-plane 23 NFFTs, each 196 taps x 4 flops per node plus an n x n FFT
        # (5 n^2 log2 n^2 flops)
        flops = nz * 23 * (196 * 4 * M + 5 * n * n * np.log2(float(n * n)))
        achieved = flops / (ms64 / fp64_steps / 1e3) / 1e12
        line["fp64_plain"] = {"value": v64, "unit": "voxel-iters/s",
                              "ms_per_step": ms64 / fp64_steps, "steps": fp64_steps,
                              "e2e": e2e64,
                              "roofline": {"bound": "fp64", "achieved": round(achieved, 4),
                                           "peak": peak64["fp64_tflops"] if peak64 else None,
                                           "unit": "TFLOP/s",
                                           "frac": round(achieved / peak64["fp64_tflops"], 4)
                                           if peak64 else None,
                                           "flops_per_step": flops,
                                           "peak_source": "measured FP64 FMA chains on this GPU "
                                                          "(nudim_gb300/bin/fp64_peak)"},
                              "fp64_peak_probe": peak64}
        line["mixed_over_fp64"] = value / v64
        line["rel_l2_mixed_vs_fp64_after_1_iteration"] = err1
        line["rel_l2_mixed_vs_fp64_after_warmup"] = err
    if small is not None:
        line["small_config"] = small
    if acc is not None:
        tot = str(r["nhio"] + r["ner"])
        rel_acc = acc["rel_l2_vs_fp64"]
        line["accuracy"] = acc
        line["rel_l2_mixed_vs_fp64_after_%s" % tot] = rel_acc["mixed"].get(tot)
        line["rel_l2_fp64_floor_after_%s" % tot] = {
            k: rel_acc["fp64_perturbed_" + k].get(tot) for k in ("1e-15", "1e-13", "6e-8")}
        line["rel_l2_mixed_fp64_hio_vs_fp64_after_%s" % tot] = rel_acc["mixed_fp64_hio"].get(tot)
        if v64 is not None:
            # the FP64-HIO schedule's time per iteration from the two measured
            # forms: nhio FP64 iterations, ner FP32 ones
            t_sched = (r["nhio"] * ms64 / fp64_steps + r["ner"] * ms_max / args.steps) / (
                r["nhio"] + r["ner"])
            line["mixed_fp64_hio"] = {"ms_per_step": t_sched, "value": ws * V / (t_sched / 1e3),
                                      "over_fp64": (ms64 / fp64_steps) / t_sched}
    if args.large:
        line["large"] = large_bench(ctx)
    elif not args.no_large_quick:
        line["large"] = large_quick(ctx)
    if args.batch_jobs > 0:
        line["batched"] = {"mixed": batched_bench(ctx, args.batch_jobs, args.steps, args.warmup,
                                                  ng.MIXED)}
    if args.serve_jobs > 0:
        line["serving"] = {"mixed": serving_bench(ctx, args.serve_jobs, args.serve_rate, ng.MIXED)}
        if args.serve_fp64:
            line["serving"]["fp64_plain"] = serving_bench(
                ctx, args.serve_fp64_jobs or args.serve_jobs,
                args.serve_fp64_rate or args.serve_rate, ng.FP64)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample(r)
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
        # fused passes (FP32 default): a gradient (2 values per voxel), 39
        # passes of 4 and an update of 3; unfused (FP64 default): 5 per inner
        # iteration
        env = os.environ.get("NUDIM_TV", "")
        fused = env == "fused" or (env != "unfused" and prec == ng.MIXED)
        per = (2 + 4 * 39 + 3) / 40.0 if fused else 5.0
        out[name] = {"ms_per_call": ms, "ms_per_inner_iteration": ms / 40,
                     "value": 40 * V / (ms / 1e3),
                     "bytes_per_inner_iteration": per * (4 if prec == ng.MIXED else 8) * V}
        log("tv %s %s: %.2f ms per 40 inner iterations" % (name, args.tv, ms))
    ctx.close()
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the accuracy leg (reduced-nz 50 HIO + 50 ER in every form)")
    ap.add_argument("--no-cfg1", action="store_true",
                    help="skip the small-configuration leg (128^3, 20 ER, TV: GPU both forms, "
                         "CPU oracle)")
    ap.add_argument("--accuracy-nz", type=int, default=16,
                    help="Z-planes of the accuracy leg's job (default 16)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain-form leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--large", action="store_true",
                    help="the large-volume configuration with the FP64 form, the FP64 "
                         "correction and the accuracy comparison (~3 min) instead of its "
                         "mixed-form timing alone")
    ap.add_argument("--no-large-quick", action="store_true",
                    help="skip the large-volume configuration's mixed-form timing")
    ap.add_argument("--batch-jobs", type=int, default=48,
                    help="jobs in the batched measurement (0: skip)")
    ap.add_argument("--serve-jobs", type=int, default=24,
                    help="jobs in the serving measurement (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=0.4,
                    help="Poisson arrivals, jobs/s (default below the measured capacity of "
                         "about 0.47 jobs/s for this job mix)")
    ap.add_argument("--serve-fp64", action="store_true", help="also serve the FP64 form")
    ap.add_argument("--serve-fp64-jobs", type=int, default=0,
                    help="jobs in the FP64 serving measurement (default: --serve-jobs)")
    ap.add_argument("--serve-fp64-rate", type=float, default=0.0,
                    help="Poisson arrivals of the FP64 serving measurement, jobs/s (default: "
                         "--serve-rate; the FP64 form's capacity is far lower)")
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
