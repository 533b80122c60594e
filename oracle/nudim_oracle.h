/*
 * nudim_oracle.h -- CPU FP64 restatement of NUDIM's reconstruction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in nudim_gb300/.  Only tests/, __graft_entry__.smoke() and
 * the cpu_baseline / --impl reference legs of bench.py may load it.  The
 * product path never links or calls it.
 *
 * Each function cites the reference file:line it restates (paths are inside
 * the gengzhi-ihep/NUDIM source tree).  NFFT3, FFTW3 and GSL are not vendored
 * by the reference; their arithmetic is restated from the published methods:
 *   - NFFT: Keiner, Kunis, Potts, "Using NFFT 3 - a software library for
 *     various nonequispaced fast Fourier transforms", ACM TOMS 36(4), 2009:
 *     Kaiser-Bessel window, cut-off m, oversampled grid n, deconvolution by
 *     the window's Fourier coefficients.
 *   - CGNR: conjugate gradients on the weighted normal equations
 *     A^H W A f = A^H W y (Bjorck, Numerical Methods for Least Squares
 *     Problems, SIAM 1996, alg. CGLS/CGNR).
 *   - FFT: any exact DFT; a mixed-radix Cooley-Tukey is used here.
 *   - RNG: MT19937 (Matsumoto & Nishimura 1998) with GSL's documented
 *     default seed convention (seed 0 -> 4357); uniform = u32 / 2^32.
 *
 * Complex arrays are interleaved (re, im) doubles.  Volumes are flat
 * [z][y][x] arrays (the reference uses double*** img[z][y][x]).
 */
#ifndef NUDIM_ORACLE_H
#define NUDIM_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sampling geometry (src/grid.c) ---- */
int  orc_equal_angle_count(double amin, double amax, double ainterval);
void orc_equal_angle_sample_2d(double amin, double amax, double ainterval, int nx,
                               double *x_out);
void orc_uniform_sample_2d(int nx, int nz, double *x_out);

/* ---- NFFT (NFFT3 nfft_init_guru / nfft_trafo / nfft_adjoint semantics) ---- */
typedef struct orc_nfft orc_nfft;
orc_nfft *orc_nfft_create(int N0, int N1, int M, const double *x);
void orc_nfft_destroy(orc_nfft *p);
void orc_nfft_trafo(orc_nfft *p, const double *f_hat, double *f);
void orc_nfft_adjoint(orc_nfft *p, const double *f, double *f_hat);
int  orc_nfft_grid_size(int N);             /* n = 2 * next_pow2(N) */
void orc_nfft_window_tables(orc_nfft *p, int *u0, int *u1, double *psi0,
                            double *psi1, double *c0, double *c1);

/* NDFT direct sums with exactly reduced phases and compensated summation. */
void orc_ndft_trafo(int N0, int N1, int M, const double *x, const double *f_hat,
                    double *f);
void orc_ndft_adjoint(int N0, int N1, int M, const double *x, const double *f,
                      double *f_hat);

/* ---- CGNR (solver_before_loop_complex + iters x solver_loop_one_step) ---- */
void orc_cgnr(orc_nfft *p, const double *y, const double *w, double *f_hat_iter,
              int iters, double *dot_z_trace);
/* Same with every NFFT output multiplied by (1 + eps N(0,1)) (test floor). */
void orc_cgnr_perturbed(orc_nfft *p, const double *y, const double *w, double *f_hat_iter,
                        int iters, double eps, unsigned long seed);

/* ---- FFT (fftw_plan_many_dft semantics, unnormalised) ---- */
void orc_fft_many(double *data, int n, int howmany, int stride, int dist, int sign);

/* ---- denoise (src/denoise.c), volumes [nz][ny][nx] ---- */
void orc_tv_discrete(const double *img, double *out, float lam, int niter,
                     int nz, int ny, int nx);
void orc_tv_discrete_height(const double *img, double *out, float lam, int niter,
                            int nz, int ny, int nx, int nheight, int ncenter);
void orc_aniso_diffusion_2d(const double *img, double *out, float lambda, float kappa,
                            int niter, int nz, int ny, int nx, int nx_bound);
void orc_show_grad_mag(const double *img, double *out, int nz, int ny, int nx);

/* ---- GSL default RNG stream (mt19937, seed 0) ---- */
void orc_mt19937_uniform(unsigned long seed, size_t n, double *out);

/* ---- full reconstruction (src/reconstruction.c:304-719) ---- */
typedef struct orc_recon_params {
    int nx, nz, np;
    double gam_min, gam_max, interval, padangle;
    int nhio, ner;
    int denoise;      /* 0 none, 1 TV, 2 DIFFUSION */
    int weight;
    int random;       /* 1: unknown samples take the values `fill` lists in (z, node)
                         order, or 10 * MT19937 uniforms when fill == NULL */
    int height, nheight, ncenter;
    int variant;      /* 0 reconstruction, 1 reconstruction_parallel */
    int cgnr_iters;   /* 10 in the reference */
    int nthreads;     /* OpenMP threads over Z-planes (1 = serial) */
    int plane_limit;  /* >0: run the NFFT+CGNR work of only this many planes
                         (bounded CPU-baseline sample); 0 = all planes */
} orc_recon_params;

/* Number of polar lines A and nodes M = A * np for the padded angle range. */
int orc_polar_lines(double gam_min, double gam_max, double interval, double padangle,
                    double *pad_min_out, double *pad_max_out);

int orc_reconstruct(const orc_recon_params *prm, const double *proj,
                    const double *fill, double *vol0_out, double *vol_out,
                    double *rhist_out);

/* Staged form: begin = setup + initial inverse (reconstruction.c:304-540),
 * iterate = n outer iterations (:545-703); times accumulate separately for
 * the per-plane NFFT+CGNR phase and the volume phases (Z-FFTs, denoise,
 * constraints). */
typedef struct orc_recon orc_recon;
orc_recon *orc_recon_begin(const orc_recon_params *prm, const double *proj,
                           const double *fill);
int orc_recon_iterate(orc_recon *R, int n, double *rhist_out);
void orc_recon_volume(const orc_recon *R, double *out);
void orc_recon_times(const orc_recon *R, double *t_planes, double *t_volume);
void orc_recon_end(orc_recon *R);

/* Individual stages, exported so tests can check intermediate arrays. */
int orc_tilt_series_fourier(int nx, int nz, int np, int nslices, const double *proj,
                            double *tomograms);
int orc_build_slices(const orc_recon_params *prm, const double *tomograms,
                     const double *fill, double *slices, int *mask);

/* ---- projection_sim -m 2D1D (src/projection_sim.c:282-405), noise-free ---- */
int orc_project_2d1d(const double *density, int nx, int ny, int nz, int np,
                     double gam_min, double gam_max, double interval,
                     double *proj_out);

#ifdef __cplusplus
}
#endif
#endif
