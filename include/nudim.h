/*
 * nudim.h -- C ABI of the GB300-native NUDIM reconstruction engine.
 *
 * The reference (gengzhi-ihep/NUDIM) has no library boundary: its hot loop is
 * inline in main() (src/reconstruction.c:545-703) and sits on the NFFT3 plan
 * and CGNR-solver API.  This header replaces that internal seam at two
 * granularities:
 *
 *   - job level: one reconstruction (the work of reconstruction.c:304-719)
 *     with every Z-plane resident on one GPU;
 *   - operator level: NFFT trafo/adjoint, the CGNR solver and the denoise
 *     stencils on device pointers plus a CUDA stream.
 *
 * Conventions
 *   - every call returns an int status: NUDIM_OK (0) or a negative NUDIM_E*;
 *     nudim_last_error() returns a message for the calling thread;
 *   - host buffers are caller-owned and copied; device buffers passed to the
 *     operator-level calls are caller-owned and are not retained;
 *   - complex arrays are interleaved (re, im) in the element type of the
 *     precision form: double for NUDIM_FP64, float for NUDIM_MIXED;
 *   - volumes are [z][y][x] with x fastest (the reference's img[z][y][x]);
 *   - a context is not thread-safe: drive it from one host thread.
 */
#ifndef NUDIM_H
#define NUDIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NUDIM_ABI_VERSION 1

enum nudim_status {
    NUDIM_OK = 0,
    NUDIM_EINVAL = -1,   /* invalid argument or unsupported size */
    NUDIM_ENOMEM = -2,   /* device or host allocation failed */
    NUDIM_ECUDA = -3,    /* CUDA / cuFFT error */
    NUDIM_ETIMEOUT = -4, /* a bounded device wait gave up */
    NUDIM_ESTATE = -5,   /* call out of order (e.g. step before projections) */
    NUDIM_EIO = -6       /* file or parse error (CLI helpers) */
};

enum nudim_precision {
    NUDIM_FP64 = 0, /* plain form: every array and operation in FP64 */
    NUDIM_MIXED = 1 /* FP32 spreading/FFT/stencils, FP64 tables + correction */
};

enum nudim_denoise {
    NUDIM_DENOISE_NONE = 0,
    NUDIM_DENOISE_TV = 1,       /* total_variation_discrete[_height] */
    NUDIM_DENOISE_DIFFUSION = 2 /* aniso_diffusion_2d */
};

enum nudim_variant {
    NUDIM_VARIANT_SERIAL = 0,  /* src/reconstruction.c behaviour */
    NUDIM_VARIANT_PARALLEL = 1 /* src/reconstruction-parallel.c behaviour */
};

typedef struct nudim_ctx nudim_ctx;
typedef struct nudim_job nudim_job;
typedef struct nudim_nfft_plan nudim_nfft_plan;

/* Reconstruction options: the reference's command line
 * (src/reconstruction.c:91-112, src/reconstruction-parallel.c:107-126). */
typedef struct nudim_job_desc {
    int nx, nz, np;         /* --nx, --nz, --pad (np and nz even) */
    double gam_min, gam_max;/* --min, --max (degrees) */
    double interval;        /* -t, measured angular step */
    double padangle;        /* --padangle, polar-grid angular step */
    int nhio, ner;          /* --nhio, --ner */
    int denoise;            /* enum nudim_denoise (NONE unless --denoise) */
    int weight;             /* --weight */
    int random;             /* --random: unknown samples from the fill */
    int height;             /* --height/--center given */
    int nheight, ncenter;   /* --height, --center */
    int variant;            /* enum nudim_variant */
    int precision;          /* enum nudim_precision */
    int cgnr_iters;         /* CGNR steps per plane (reference: 10; 0 -> 10) */
    int correct_every;      /* NUDIM_MIXED: k > 0, every k-th iteration is an FP64
                               residual check / corrective iteration; k < 0, every
                               HIO iteration runs in FP64 (from the FP64 initial
                               inverse) and only ER iterations in FP32; 0: never */
} nudim_job_desc;

/* ------------------------------------------------------------------ */
/* context                                                             */
/* ------------------------------------------------------------------ */
const char *nudim_last_error(void);
int nudim_abi_version(void);

/* Context flags. */
#define NUDIM_CTX_GRID_NFFT 1u /* NFFT through an n0 x n1 grid in HBM + cuFFT (cross-check
                                  path); the default keeps the grid on chip (fused) */
#define NUDIM_CTX_AUTOTUNE 2u  /* the first fused NFFT plan of each geometry (N0, N1, M,
                                  precision) times one trafo + adjoint for each trafo
                                  column width and planes per spreading CTA and keeps
                                  the fastest for the context's later plans; no
                                  reference counterpart (NFFT3 plans have no such
                                  choice) */

/* Create a context on CUDA device `device`.  flags: 0 or NUDIM_CTX_* bits. */
int nudim_ctx_create(int device, unsigned flags, nudim_ctx **out);
int nudim_ctx_destroy(nudim_ctx *ctx);
/* CUDA stream (cudaStream_t) the context launches job work on. */
void *nudim_ctx_stream(nudim_ctx *ctx);
/* Tracing (no counterpart in the reference, which only prints MPI_Wtime
 * totals, reconstruction-parallel.c:881-883): per-kernel-class CUDA-event
 * timing of the context's launches.  enable != 0 starts timing and clears
 * the totals; nudim_ctx_profile_read synchronises and returns, for kernel
 * class k (0 .. nudim_profile_kernel_count()-1), the summed device time,
 * the number of timed launches and the algorithmic bytes they move. */
int nudim_ctx_profile(nudim_ctx *ctx, int enable);
int nudim_ctx_profile_read(nudim_ctx *ctx, int k, double *total_ms, long long *launches,
                           double *bytes);
int nudim_profile_kernel_count(void);
const char *nudim_profile_kernel_name(int k);
/* Kernels launched by this library in this process so far. */
unsigned long long nudim_launch_count(void);

/* Bytes of device memory a job with this descriptor keeps resident. */
int nudim_job_footprint(const nudim_job_desc *desc, size_t *bytes);

/* ------------------------------------------------------------------ */
/* job level: replaces the body of src/reconstruction.c:304-719        */
/* ------------------------------------------------------------------ */

/* Validate the descriptor (reconstruction.c:245-293 rules plus even sizes),
 * build the polar node set (grid.c:78-97), the Kaiser-Bessel and
 * deconvolution tables, the CGNR weights (reconstruction.c:415-426) and
 * allocate every device buffer of the job. */
int nudim_job_create(nudim_ctx *ctx, const nudim_job_desc *desc, nudim_job **out);
int nudim_job_destroy(nudim_job *job);

/* Optional: values for the unknown Fourier samples when desc->random is set,
 * listed in (z, node) order as reconstruction.c:437-484 draws them
 * (gsl_rng_uniform()*10).  Without this call a random job draws them from
 * the library's MT19937 stream (seed 4357, GSL's default). */
int nudim_job_import_fill(nudim_job *job, const double *fill, size_t n);

/* Upload the measured tilt series (host FP64, [tilt][z][x], tilt j at
 * gam_min + j*interval) and run the setup stages: tilt-series NFFT
 * (reconstruction.c:307-367), reorder/mask/fill (:437-484) and the initial
 * inverse NFFT + backward Z-FFT (:489-540). */
int nudim_job_set_projections(nudim_job *job, const double *proj, size_t n);

/* Run `iters` outer HIO/ER iterations (reconstruction.c:545-703) of each
 * job; the iteration counter of each job continues from where it stopped
 * and never passes nhio+ner.  Iterations are queued round-robin over the
 * jobs, each on its own stream, so they overlap on the device; the call
 * returns when the work is queued (sync with nudim_job_sync, nudim_ctx_sync
 * or by reading results).  A NUDIM_MIXED job's check iteration (see
 * nudim_job_corrections; NUDIM_CORRECT_TOL > 0) first queues the residual
 * check and is itself queued once the check's result reaches the host: the
 * other jobs' iterations are queued meanwhile, and the call waits on the host
 * only when every iteration it has left waits on a check. */
int nudim_step(nudim_ctx *ctx, nudim_job *const *jobs, int njobs, int iters);
/* Wait for all queued work of every job on the context's device. */
int nudim_ctx_sync(nudim_ctx *ctx);
/* Each job owns a CUDA stream (its allocations, transforms and kernels are
 * ordered on it), so the jobs of one nudim_step call overlap on the device. */
void *nudim_job_stream(nudim_job *job);
int nudim_job_sync(nudim_job *job);

/* Copy the current volume to host FP64.  crop=0: full nz*np*np volume
 * (recovered-0.txt layout); crop=1: central nx*nx crop of every plane in
 * recovered.txt order (reconstruction.c:706-719), nz*nx*nx values. */
int nudim_job_get_volume(nudim_job *job, double *out, size_t n, int crop);
/* Volume after the initial inverse NFFT (recovered-0.txt, full). */
int nudim_job_get_initial_volume(nudim_job *job, double *out, size_t n);
/* R-factor history sqrt(diff1/diff2) per finished iteration
 * (reconstruction.c:603-604).  *count receives the number written. */
int nudim_job_get_rfactor(nudim_job *job, double *hist, int cap, int *count);
int nudim_job_iterations_done(nudim_job *job, int *done);
/* FP64 iterations a NUDIM_MIXED job has run (desc.correct_every = k > 0:
 * every k-th iteration checks the measured-slice mismatch R of the current
 * volume in FP32 and FP64 and runs the iteration in FP64 when they differ
 * by more than the relative tolerance NUDIM_CORRECT_TOL (environment; 0, the
 * default, corrects at every check); k < 0: every HIO iteration).
 * Consecutive FP64 iterations keep the volume in FP64.  No reference
 * counterpart. */
int nudim_job_corrections(nudim_job *job, int *count);
/* Capture the volume before and after denoising at outer iteration `nn`
 * (the reference's grad_before/grad_after dumps).  Host buffers of
 * nz*np*np doubles each stay owned by the caller; pass nn < 0 to disable. */
int nudim_job_set_denoise_dump(nudim_job *job, int nn, double *before, double *after);

/* ------------------------------------------------------------------ */
/* serving: continuous batching of reconstruction jobs (no counterpart */
/* in the reference, which reconstructs one tomogram per process)     */
/* ------------------------------------------------------------------ */
typedef struct nudim_server nudim_server;

/* A request loop on its own host thread: queued requests are admitted while
 * their device-memory footprint (nudim_job_footprint plus workspace) fits
 * mem_budget and fewer than max_active jobs run; admitted jobs stay
 * resident, their outer iterations are queued round-robin on per-job
 * streams (at most two in flight each) so they overlap on the device, and a
 * finished job's volume is copied out and its memory released. */
int nudim_server_create(nudim_ctx *ctx, size_t mem_budget, int max_active, nudim_server **out);
/* Thread-safe; copies the tilt series; the arrival time is stamped here. */
int nudim_server_submit(nudim_server *s, const nudim_job_desc *desc, const double *proj,
                        size_t n, long long *ticket);
/* Block until the ticket's job is done; copy its volume (crop as in
 * nudim_job_get_volume; vol may be NULL) and its arrival-to-result latency. */
int nudim_server_wait(nudim_server *s, long long ticket, double *vol, size_t n, int crop,
                      double *latency_s);
/* Completed jobs, median and 99th-percentile latency (s), completed jobs per
 * second from the first arrival to the last completion. */
int nudim_server_stats(nudim_server *s, long long *completed, double *p50_s, double *p99_s,
                       double *jobs_per_s);
/* Finish every submitted job, then stop the loop. */
int nudim_server_destroy(nudim_server *s);

/* projection_sim -m 2D1D (src/projection_sim.c:282-405) on the GPU, FP64:
 * density [nz][ny][nx] (host) -> tilt series [tilt][nz][np] (host), tilts
 * gam_min + j*interval, values Re(slice)/(np*nz) as the reference writes
 * them.  snr > 0 adds Gaussian noise of std(slice)/snr per tilt
 * (projection_sim.c:45-67) from the library's seeded generator (MT19937 +
 * Box-Muller; GSL's Gaussian sampler is not reproduced). */
int nudim_project_2d1d(nudim_ctx *ctx, const double *density, int nx, int ny, int nz, int np,
                       double gam_min, double gam_max, double interval, double snr,
                       unsigned long seed, double *proj_out, size_t n_out);

/* projection_sim -m DFT (src/projection_sim.c:516-600) on the GPU, FP64:
 * the same arguments and output as nudim_project_2d1d, the Fourier samples
 * computed as the reference's exact sums over every voxel with its phase
 * cos(2 PI t) - i sin(2 PI t), PI = 3.1415926 (src/grid.h:11), and the 3D
 * method's shifts of both axes around the 2D inverse FFT.  -m 3D
 * (src/projection_sim.c:409-514) samples the same transform with a 3D NFFT;
 * its output equals nudim_project_2d1d's to the NFFT's accuracy. */
int nudim_project_dft(nudim_ctx *ctx, const double *density, int nx, int ny, int nz, int np,
                      double gam_min, double gam_max, double interval, double snr,
                      unsigned long seed, double *proj_out, size_t n_out);

/* ------------------------------------------------------------------ */
/* operator level (device pointers, caller stream)                     */
/* ------------------------------------------------------------------ */

/* nfft_init_guru(&p, 2, {N0,N1}, M, {n0,n1}, 6, PRE_PHI_HUT|PRE_FULL_PSI|...)
 * (reconstruction.c:319-331, 393-405): x holds 2*M host doubles in
 * [-1/2,1/2), dimension 0 first.  n = 2*next_pow2(N) per dimension, m = 6. */
int nudim_nfft_plan_create(nudim_ctx *ctx, int N0, int N1, int M, const double *x,
                           int precision, nudim_nfft_plan **out);
int nudim_nfft_plan_destroy(nudim_nfft_plan *plan);
/* The plan's fused-path choice: trafo column-block width and Z-planes per
 * spreading CTA (both 0 on the grid path).  No reference counterpart. */
int nudim_nfft_plan_tuning(nudim_nfft_plan *plan, int *trafo_cols, int *spread_planes);

/* nfft_trafo (reconstruction.c:361, 571) on `nplanes` planes:
 * f[p][j] = sum_k f_hat[p][k] exp(-2 pi i k.x_j); f_hat planes are N0*N1
 * complex (row-major, centred index), f planes are M complex. */
int nudim_nfft_trafo(nudim_nfft_plan *plan, int nplanes, const void *f_hat, void *f,
                     void *stream);
/* nfft_adjoint (inside the CGNR solver): f_hat[p][k] = sum_j f[p][j] exp(+2 pi i k.x_j). */
int nudim_nfft_adjoint(nudim_nfft_plan *plan, int nplanes, const void *f, void *f_hat,
                       void *stream);

/* solver_init_advanced_complex(CGNR[|PRECOMPUTE_WEIGHT]) +
 * solver_before_loop_complex + iters x solver_loop_one_step_complex
 * (reconstruction.c:407-413, 506-509, 592-595) on `nplanes` independent
 * planes: y[p] (M complex), w (M real, NULL for unweighted, shared by all
 * planes), f_hat_iter[p] (N0*N1 complex, start value in, solution out). */
int nudim_cgnr(nudim_nfft_plan *plan, int nplanes, const void *y, const void *w,
               void *f_hat_iter, int iters, void *stream);

/* total_variation_discrete[_height] (denoise.c:67-249), in place on a
 * [nz][ny][nx] volume of the plan precision's real type.  height != 0
 * restricts to rows y in [(2c-h)/2, (2c+h)/2]. */
int nudim_tv(nudim_ctx *ctx, int precision, void *vol, int nz, int ny, int nx, float lam,
             int niter, int height, int nheight, int ncenter, void *stream);

/* nudim_tv without any device allocation.  No counterpart in the reference:
 * it serves callers that cannot call cudaMalloc (a host whose memory
 * manager owns the whole device, or a loop that must avoid the implicit
 * synchronisation of cudaMalloc/cudaFree).  Same semantics and kernels as
 * nudim_tv on the current CUDA device; the scratch (gradient field and sums)
 * is one fixed 32 MiB (33554432-byte) device array inside this library,
 * present on every GPU that loads it until the process exits.  A volume
 * needs round_up(8 * (K + 4), 256) + S * nz*ny*nx bytes of it, with
 * K = 2 * ceil(nx/32) * ceil(ny/16) * nz + 2 partial sums and S = 8 (FP64)
 * or 4 (FP32); for planes that are whole 32 x 16 tiles that is about
 * 4.1 million FP64 or 8.3 million FP32 voxels (e.g. FP32 127 x 256 x 256),
 * while thin planes (nx or ny far below a tile) need far more partial sums
 * per voxel.  Larger volumes return NUDIM_EINVAL.  The first call in each
 * CUDA context on a device looks up the array's device address; make that
 * first call before any stream capture.  All calls share the array: calls
 * whose work overlaps on a GPU race and must be serialised by the caller. */
int nudim_tv_noalloc(int precision, void *vol, int nz, int ny, int nx, float lam, int niter,
                     int height, int nheight, int ncenter, void *stream);

/* aniso_diffusion_2d (denoise.c:320-378), in place, Gauss-Seidel order per
 * Z-plane.  nx_bound is the value the reference compares the column index
 * with (its "nx" argument, the number of Z-planes in reconstruction.c:627);
 * a read one past the row is defined as 0.0. */
int nudim_diffusion2d(nudim_ctx *ctx, int precision, void *vol, int nz, int ny, int nx,
                      int nx_bound, float lambda, float kappa, int niter, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NUDIM_H */
