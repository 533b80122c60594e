/*
 * nudim_oracle.c -- CPU FP64 restatement of NUDIM's reconstruction path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): see
 * nudim_oracle.h for who may load it and which published methods stand in
 * for the un-vendored NFFT3 / FFTW3 / GSL arithmetic.
 *
 * Floating point: build with -ffp-contract=off so that x86-64 and aarch64
 * produce identical bits (the reference's own Makefile builds with gcc -O3,
 * which on x86-64 without -march emits no fused multiply-add either).
 */
#include "nudim_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* src/grid.h:11 -- the reference's truncated constant, used for node angles,
 * CGNR weights and nothing else.  The NFFT window uses the true pi. */
#define REF_PI 3.1415926
#define TRUE_PI 3.14159265358979323846

/* ===================================================================== */
/* Sampling geometry                                                      */
/* ===================================================================== */

/* src/grid.c:61-76 (grid_slice_2D): radius by repeated addition of 1/nx,
 * node = (r sin g, r cos g), angle in degrees converted with PI=3.1415926. */
static void slice_2d(int nx, double gama, double *x)
{
    double interval = 1.0 / nx;
    double x0 = -0.5 - interval;
    for (int i = 0; i < nx; i++) {
        x0 += interval;
        x[2 * i + 0] = x0 * sin(gama / 180 * REF_PI);
        x[2 * i + 1] = x0 * cos(gama / 180 * REF_PI);
    }
}

/* src/grid.c:84 */
int orc_equal_angle_count(double amin, double amax, double ainterval)
{
    return (int)((amax - amin) / ainterval + 0.5) + 1;
}

/* src/grid.c:78-97: angle by repeated addition starting at amin - interval. */
void orc_equal_angle_sample_2d(double amin, double amax, double ainterval, int nx,
                               double *x)
{
    int ns = orc_equal_angle_count(amin, amax, ainterval);
    double angle = amin - ainterval;
    for (int i = 0; i < ns; i++) {
        angle += ainterval;
        slice_2d(nx, angle, x + (size_t)i * nx * 2);
    }
}

/* src/grid.c:100-133: X fastest, Z slowest, both by repeated addition. */
void orc_uniform_sample_2d(int nx, int nz, double *x)
{
    double ix = 1.0 / nx, iz = 1.0 / nz;
    double z0 = -0.5 - iz;
    for (int j = 0; j < nz; j++) {
        z0 += iz;
        double x0 = -0.5 - ix;
        for (int i = 0; i < nx; i++) {
            x0 += ix;
            x[2 * ((size_t)j * nx + i) + 0] = x0;
            x[2 * ((size_t)j * nx + i) + 1] = z0;
        }
    }
}

/* src/reconstruction.c:372-384: padded angle range and line count. */
int orc_polar_lines(double gam_min, double gam_max, double interval, double padangle,
                    double *pad_min_out, double *pad_max_out)
{
    (void)gam_max;
    int ntmp = (int)((-90 - gam_min) / interval);
    double pad_min = gam_min + ntmp * interval;
    ntmp = (int)((90 - gam_min) / interval);
    double pad_max = gam_min + ntmp * interval;
    if (pad_min_out) *pad_min_out = pad_min;
    if (pad_max_out) *pad_max_out = pad_max;
    return orc_equal_angle_count(pad_min, pad_max, padangle);
}

/* ===================================================================== */
/* FFT: mixed-radix decimation in time, unnormalised, FFTW sign convention */
/* ===================================================================== */

typedef struct {
    int n;
    cplx *tw; /* exp(sign * 2 pi i t / n), t < n */
} fft_tw;

static void fft_tw_init(fft_tw *t, int n, int sign)
{
    t->n = n;
    t->tw = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int k = 0; k < n; k++) {
        double a = 2.0 * TRUE_PI * (double)k / (double)n;
        t->tw[k] = cos(a) + (double)sign * sin(a) * I;
    }
}

static int smallest_factor(int n)
{
    if (n % 4 == 0) return 4;
    if (n % 2 == 0) return 2;
    for (int p = 3; p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

/* out[k] = sum_t in[t*stride] * W^(t k),  W = tw of length N, step = N / n. */
static void fft_rec(const cplx *in, int stride, cplx *out, int n, const fft_tw *T, int step)
{
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; r++)
        fft_rec(in + (size_t)r * stride, stride * p, out + (size_t)r * m, m, T, step * p);
    cplx tmp[64];
    cplx *buf = (p <= 64) ? tmp : (cplx *)malloc(sizeof(cplx) * (size_t)p);
    int N = T->n;
    for (int k = 0; k < m; k++) {
        for (int r = 0; r < p; r++) {
            /* twiddle W_n^{r k} applied to sub-transform r */
            buf[r] = out[(size_t)r * m + k] * T->tw[((long)r * k * step) % N];
        }
        for (int q = 0; q < p; q++) {
            cplx s = 0;
            for (int r = 0; r < p; r++)
                s += buf[r] * T->tw[((long)r * q * m * step) % N];
            out[(size_t)q * m + k] = s;
        }
    }
    if (buf != tmp) free(buf);
}

static void fft_1d(cplx *work_in, cplx *work_out, int n, const fft_tw *T)
{
    fft_rec(work_in, 1, work_out, n, T, 1);
}

/* fftw_plan_many_dft(1, &n, howmany, data, NULL, stride, dist, data, NULL,
 * stride, dist, sign): reconstruction.c:521-523, 556-559, 607-610. */
void orc_fft_many(double *data_d, int n, int howmany, int stride, int dist, int sign)
{
    cplx *data = (cplx *)data_d;
    fft_tw T;
    fft_tw_init(&T, n, sign < 0 ? -1 : 1);
    /* independent transforms: threads cannot change any result */
#pragma omp parallel
    {
        cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)n);
        cplx *b = (cplx *)malloc(sizeof(cplx) * (size_t)n);
#pragma omp for schedule(static)
        for (int h = 0; h < howmany; h++) {
            cplx *base = data + (size_t)h * dist;
            for (int t = 0; t < n; t++) a[t] = base[(size_t)t * stride];
            fft_1d(a, b, n, &T);
            for (int t = 0; t < n; t++) base[(size_t)t * stride] = b[t];
        }
        free(a);
        free(b);
    }
    free(T.tw);
}

/* 2D FFT of a row-major n0 x n1 grid with precomputed twiddles. */
static void fft_2d(cplx *g, int n0, int n1, const fft_tw *T0, const fft_tw *T1, cplx *a,
                   cplx *b)
{
    for (int r = 0; r < n0; r++) {
        cplx *row = g + (size_t)r * n1;
        memcpy(a, row, sizeof(cplx) * (size_t)n1);
        fft_1d(a, row, n1, T1);
    }
    for (int c = 0; c < n1; c++) {
        for (int r = 0; r < n0; r++) a[r] = g[(size_t)r * n1 + c];
        fft_1d(a, b, n0, T0);
        for (int r = 0; r < n0; r++) g[(size_t)r * n1 + c] = b[r];
    }
}

/* ===================================================================== */
/* NFFT with the Kaiser-Bessel window (published method, m = 6)          */
/* ===================================================================== */

#define NFFT_M 6
#define NFFT_W (2 * NFFT_M + 2)

struct orc_nfft {
    int N0, N1, n0, n1, M;
    double b0, b1;
    double *x;
    int *u0, *u1;
    double *psi0, *psi1; /* M x NFFT_W */
    double *c0, *c1;     /* N0, N1: 1 / phi_hat */
    fft_tw Tf0, Tf1, Tb0, Tb1;
};

int orc_nfft_grid_size(int N)
{
    /* reconstruction.c:316-317, 390-391: n = 2 * nfft_next_power_of_2(N) */
    int p = 1;
    while (p < N) p <<= 1;
    return 2 * p;
}

/* Modified Bessel function I0 by its power series; all terms positive, so
 * the sum is accurate to a few ulp for the arguments used here (< 40). */
static double bessel_i0(double x)
{
    double q = 0.25 * x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; k++) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < sum * 1e-18) break;
    }
    return sum;
}

/* KB window phi(x) with dn = x * n (distance in grid cells). */
static double kb_phi(double dn, double b)
{
    double m2 = (double)NFFT_M * NFFT_M;
    double a = m2 - dn * dn;
    if (a > 0) {
        double s = sqrt(a);
        return sinh(b * s) / (TRUE_PI * s);
    } else if (a < 0) {
        double s = sqrt(-a);
        return sin(b * s) / (TRUE_PI * s);
    }
    return b / TRUE_PI;
}

/* n * phi_hat(k): Fourier coefficient of the window (without the 1/n). */
static double kb_phi_hat(int k, int n, double b)
{
    double t = 2.0 * TRUE_PI * (double)k / (double)n;
    return bessel_i0((double)NFFT_M * sqrt(b * b - t * t));
}

orc_nfft *orc_nfft_create(int N0, int N1, int M, const double *x)
{
    orc_nfft *p = (orc_nfft *)calloc(1, sizeof(orc_nfft));
    p->N0 = N0;
    p->N1 = N1;
    p->M = M;
    p->n0 = orc_nfft_grid_size(N0);
    p->n1 = orc_nfft_grid_size(N1);
    p->b0 = TRUE_PI * (2.0 - 1.0 / ((double)p->n0 / (double)N0));
    p->b1 = TRUE_PI * (2.0 - 1.0 / ((double)p->n1 / (double)N1));
    p->x = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    memcpy(p->x, x, sizeof(double) * 2 * (size_t)M);
    p->u0 = (int *)malloc(sizeof(int) * (size_t)M);
    p->u1 = (int *)malloc(sizeof(int) * (size_t)M);
    p->psi0 = (double *)malloc(sizeof(double) * (size_t)M * NFFT_W);
    p->psi1 = (double *)malloc(sizeof(double) * (size_t)M * NFFT_W);
    for (int j = 0; j < M; j++) {
        for (int t = 0; t < 2; t++) {
            int n = t ? p->n1 : p->n0;
            double b = t ? p->b1 : p->b0;
            double xn = x[2 * j + t] * (double)n;
            int u = (int)floor(xn) - NFFT_M;
            (t ? p->u1 : p->u0)[j] = u;
            double *psi = (t ? p->psi1 : p->psi0) + (size_t)j * NFFT_W;
            for (int s = 0; s < NFFT_W; s++) psi[s] = kb_phi(xn - (double)(u + s), b);
        }
    }
    p->c0 = (double *)malloc(sizeof(double) * (size_t)N0);
    p->c1 = (double *)malloc(sizeof(double) * (size_t)N1);
    for (int k = 0; k < N0; k++) p->c0[k] = 1.0 / kb_phi_hat(k - N0 / 2, p->n0, p->b0);
    for (int k = 0; k < N1; k++) p->c1[k] = 1.0 / kb_phi_hat(k - N1 / 2, p->n1, p->b1);
    fft_tw_init(&p->Tf0, p->n0, -1);
    fft_tw_init(&p->Tf1, p->n1, -1);
    fft_tw_init(&p->Tb0, p->n0, +1);
    fft_tw_init(&p->Tb1, p->n1, +1);
    return p;
}

void orc_nfft_destroy(orc_nfft *p)
{
    if (!p) return;
    free(p->x);
    free(p->u0);
    free(p->u1);
    free(p->psi0);
    free(p->psi1);
    free(p->c0);
    free(p->c1);
    free(p->Tf0.tw);
    free(p->Tf1.tw);
    free(p->Tb0.tw);
    free(p->Tb1.tw);
    free(p);
}

void orc_nfft_window_tables(orc_nfft *p, int *u0, int *u1, double *psi0, double *psi1,
                            double *c0, double *c1)
{
    size_t M = (size_t)p->M;
    if (u0) memcpy(u0, p->u0, sizeof(int) * M);
    if (u1) memcpy(u1, p->u1, sizeof(int) * M);
    if (psi0) memcpy(psi0, p->psi0, sizeof(double) * M * NFFT_W);
    if (psi1) memcpy(psi1, p->psi1, sizeof(double) * M * NFFT_W);
    if (c0) memcpy(c0, p->c0, sizeof(double) * (size_t)p->N0);
    if (c1) memcpy(c1, p->c1, sizeof(double) * (size_t)p->N1);
}

typedef struct {
    cplx *g, *a, *b;
} nfft_ws;

static void ws_init(nfft_ws *w, const orc_nfft *p)
{
    int nm = p->n0 > p->n1 ? p->n0 : p->n1;
    w->g = (cplx *)malloc(sizeof(cplx) * (size_t)p->n0 * p->n1);
    w->a = (cplx *)malloc(sizeof(cplx) * (size_t)nm);
    w->b = (cplx *)malloc(sizeof(cplx) * (size_t)nm);
}

static void ws_free(nfft_ws *w)
{
    free(w->g);
    free(w->a);
    free(w->b);
}

/* index modulo the oversampled grid size (a power of two) */
static inline int wrap(int l, int n) { return l & (n - 1); }

/* nfft_trafo (reconstruction.c:361, 571): f_j = sum_k f_hat_k exp(-2 pi i k x_j).
 * D: deconvolve + place at k mod n; F: forward FFT; B: window interpolation. */
static void nfft_trafo_ws(const orc_nfft *p, nfft_ws *w, const cplx *f_hat, cplx *f)
{
    int N0 = p->N0, N1 = p->N1, n0 = p->n0, n1 = p->n1;
    memset(w->g, 0, sizeof(cplx) * (size_t)n0 * n1);
    for (int a = 0; a < N0; a++) {
        int l0 = wrap(a - N0 / 2, n0);
        for (int c = 0; c < N1; c++) {
            int l1 = wrap(c - N1 / 2, n1);
            w->g[(size_t)l0 * n1 + l1] = f_hat[(size_t)a * N1 + c] * (p->c0[a] * p->c1[c]);
        }
    }
    fft_2d(w->g, n0, n1, &p->Tf0, &p->Tf1, w->a, w->b);
    for (int j = 0; j < p->M; j++) {
        const double *s0 = p->psi0 + (size_t)j * NFFT_W;
        const double *s1 = p->psi1 + (size_t)j * NFFT_W;
        cplx acc = 0;
        for (int t0 = 0; t0 < NFFT_W; t0++) {
            const cplx *row = w->g + (size_t)wrap(p->u0[j] + t0, n0) * n1;
            cplx ra = 0;
            for (int t1 = 0; t1 < NFFT_W; t1++) ra += s1[t1] * row[wrap(p->u1[j] + t1, n1)];
            acc += s0[t0] * ra;
        }
        f[j] = acc;
    }
}

/* nfft_adjoint (inside the CGNR solver): f_hat_k = sum_j f_j exp(+2 pi i k x_j).
 * B^T: spread; F^H: backward FFT; D: crop + deconvolve. */
static void nfft_adjoint_ws(const orc_nfft *p, nfft_ws *w, const cplx *f, cplx *f_hat)
{
    int N0 = p->N0, N1 = p->N1, n0 = p->n0, n1 = p->n1;
    memset(w->g, 0, sizeof(cplx) * (size_t)n0 * n1);
    for (int j = 0; j < p->M; j++) {
        const double *s0 = p->psi0 + (size_t)j * NFFT_W;
        const double *s1 = p->psi1 + (size_t)j * NFFT_W;
        for (int t0 = 0; t0 < NFFT_W; t0++) {
            cplx *row = w->g + (size_t)wrap(p->u0[j] + t0, n0) * n1;
            cplx v = s0[t0] * f[j];
            for (int t1 = 0; t1 < NFFT_W; t1++) row[wrap(p->u1[j] + t1, n1)] += s1[t1] * v;
        }
    }
    fft_2d(w->g, n0, n1, &p->Tb0, &p->Tb1, w->a, w->b);
    for (int a = 0; a < N0; a++) {
        int l0 = wrap(a - N0 / 2, n0);
        for (int c = 0; c < N1; c++) {
            int l1 = wrap(c - N1 / 2, n1);
            f_hat[(size_t)a * N1 + c] = w->g[(size_t)l0 * n1 + l1] * (p->c0[a] * p->c1[c]);
        }
    }
}

void orc_nfft_trafo(orc_nfft *p, const double *f_hat, double *f)
{
    nfft_ws w;
    ws_init(&w, p);
    nfft_trafo_ws(p, &w, (const cplx *)f_hat, (cplx *)f);
    ws_free(&w);
}

void orc_nfft_adjoint(orc_nfft *p, const double *f, double *f_hat)
{
    nfft_ws w;
    ws_init(&w, p);
    nfft_adjoint_ws(p, &w, (const cplx *)f, (cplx *)f_hat);
    ws_free(&w);
}

/* ---------------------------------------------------------------------- */
/* NDFT direct sums (known answer for the NFFT).                           */
/* ---------------------------------------------------------------------- */

/* exp(sgn * 2 pi i k x) with k*x split exactly (fma residual) and reduced
 * modulo 1 before the trigonometric call. */
static void phase_table(int N, double x, int sgn, cplx *e)
{
    for (int a = 0; a < N; a++) {
        double k = (double)(a - N / 2);
        double pr = k * x;
        double er = fma(k, x, -pr);
        double fr = pr - nearbyint(pr);
        double arg = fr + er;
        double ang = 2.0 * TRUE_PI * arg;
        e[a] = cos(ang) + (double)sgn * sin(ang) * I;
    }
}

typedef struct {
    double s, c;
} kahan;
static inline void kadd(kahan *k, double v)
{
    double t = k->s + v;
    if (fabs(k->s) >= fabs(v))
        k->c += (k->s - t) + v;
    else
        k->c += (v - t) + k->s;
    k->s = t;
}

void orc_ndft_trafo(int N0, int N1, int M, const double *x, const double *f_hat_d,
                    double *f_d)
{
    const cplx *f_hat = (const cplx *)f_hat_d;
    cplx *f = (cplx *)f_d;
    cplx *e0 = (cplx *)malloc(sizeof(cplx) * (size_t)N0);
    cplx *e1 = (cplx *)malloc(sizeof(cplx) * (size_t)N1);
    for (int j = 0; j < M; j++) {
        phase_table(N0, x[2 * j], -1, e0);
        phase_table(N1, x[2 * j + 1], -1, e1);
        kahan re = {0, 0}, im = {0, 0};
        for (int a = 0; a < N0; a++)
            for (int c = 0; c < N1; c++) {
                cplx t = f_hat[(size_t)a * N1 + c] * (e0[a] * e1[c]);
                kadd(&re, creal(t));
                kadd(&im, cimag(t));
            }
        f[j] = (re.s + re.c) + (im.s + im.c) * I;
    }
    free(e0);
    free(e1);
}

void orc_ndft_adjoint(int N0, int N1, int M, const double *x, const double *f_d,
                      double *f_hat_d)
{
    const cplx *f = (const cplx *)f_d;
    cplx *f_hat = (cplx *)f_hat_d;
    size_t NN = (size_t)N0 * N1;
    kahan *re = (kahan *)calloc(NN, sizeof(kahan));
    kahan *im = (kahan *)calloc(NN, sizeof(kahan));
    cplx *e0 = (cplx *)malloc(sizeof(cplx) * (size_t)N0);
    cplx *e1 = (cplx *)malloc(sizeof(cplx) * (size_t)N1);
    for (int j = 0; j < M; j++) {
        phase_table(N0, x[2 * j], +1, e0);
        phase_table(N1, x[2 * j + 1], +1, e1);
        for (int a = 0; a < N0; a++)
            for (int c = 0; c < N1; c++) {
                cplx t = f[j] * (e0[a] * e1[c]);
                kadd(&re[(size_t)a * N1 + c], creal(t));
                kadd(&im[(size_t)a * N1 + c], cimag(t));
            }
    }
    for (size_t k = 0; k < NN; k++)
        f_hat[k] = (re[k].s + re[k].c) + (im[k].s + im[k].c) * I;
    free(re);
    free(im);
    free(e0);
    free(e1);
}

/* ===================================================================== */
/* CGNR (NFFT3 solver with CGNR flag, optional PRECOMPUTE_WEIGHT)         */
/* reconstruction.c:506-509, 592-595                                      */
/* ===================================================================== */

typedef struct {
    cplx *r, *v, *z, *p, *wr;
    nfft_ws nw;
    double noise;   /* test hook: relative noise on every NFFT output (0: off) */
    uint64_t rng;
} cg_ws;

/* splitmix64 + Box-Muller: Gaussian noise for the perturbation hook */
static double gauss(uint64_t *s)
{
    uint64_t z[2];
    for (int q = 0; q < 2; q++) {
        uint64_t x = (*s += 0x9e3779b97f4a7c15ull);
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
        z[q] = x ^ (x >> 31);
    }
    double u1 = ((double)(z[0] >> 11) + 1.0) / 9007199254740993.0;
    double u2 = (double)(z[1] >> 11) / 9007199254740992.0;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * TRUE_PI * u2);
}

static void perturb(cg_ws *c, cplx *v, size_t n)
{
    if (!c->noise) return;
    for (size_t i = 0; i < n; i++) v[i] *= 1.0 + c->noise * gauss(&c->rng);
}

static void cg_init(cg_ws *c, const orc_nfft *p)
{
    size_t M = (size_t)p->M, N = (size_t)p->N0 * p->N1;
    c->noise = 0;
    c->rng = 0;
    c->r = (cplx *)malloc(sizeof(cplx) * M);
    c->v = (cplx *)malloc(sizeof(cplx) * M);
    c->wr = (cplx *)malloc(sizeof(cplx) * M);
    c->z = (cplx *)malloc(sizeof(cplx) * N);
    c->p = (cplx *)malloc(sizeof(cplx) * N);
    ws_init(&c->nw, p);
}

static void cg_free(cg_ws *c)
{
    free(c->r);
    free(c->v);
    free(c->wr);
    free(c->z);
    free(c->p);
    ws_free(&c->nw);
}

static inline double cabs2(cplx a) { return creal(a) * creal(a) + cimag(a) * cimag(a); }

/* before_loop: r = y - A f; z = A^H W r; p = z.
 * step: v = A p; alpha = |z|^2 / (v^H W v); f += alpha p; r -= alpha v;
 *       z' = A^H W r; beta = |z'|^2 / |z|^2; p = beta p + z'. */
static void cgnr_ws(const orc_nfft *pl, cg_ws *c, const cplx *y, const double *w, cplx *f,
                    int iters, double *trace)
{
    int M = pl->M, N = pl->N0 * pl->N1;
    nfft_trafo_ws(pl, &c->nw, f, c->v);
    perturb(c, c->v, M);
    for (int j = 0; j < M; j++) {
        c->r[j] = y[j] - c->v[j];
        c->wr[j] = w ? w[j] * c->r[j] : c->r[j];
    }
    nfft_adjoint_ws(pl, &c->nw, c->wr, c->z);
    perturb(c, c->z, N);
    double dot_z = 0;
    for (int k = 0; k < N; k++) {
        dot_z += cabs2(c->z[k]);
        c->p[k] = c->z[k];
    }
    if (trace) trace[0] = dot_z;
    for (int it = 0; it < iters; it++) {
        nfft_trafo_ws(pl, &c->nw, c->p, c->v);
        perturb(c, c->v, M);
        double dot_v = 0;
        for (int j = 0; j < M; j++) dot_v += (w ? w[j] : 1.0) * cabs2(c->v[j]);
        double alpha = dot_z / dot_v;
        for (int k = 0; k < N; k++) f[k] += alpha * c->p[k];
        for (int j = 0; j < M; j++) {
            c->r[j] -= alpha * c->v[j];
            c->wr[j] = w ? w[j] * c->r[j] : c->r[j];
        }
        nfft_adjoint_ws(pl, &c->nw, c->wr, c->z);
        perturb(c, c->z, N);
        double dot_z_new = 0;
        for (int k = 0; k < N; k++) dot_z_new += cabs2(c->z[k]);
        double beta = dot_z_new / dot_z;
        dot_z = dot_z_new;
        for (int k = 0; k < N; k++) c->p[k] = beta * c->p[k] + c->z[k];
        if (trace) trace[it + 1] = dot_z;
    }
}

void orc_cgnr(orc_nfft *p, const double *y, const double *w, double *f_hat_iter, int iters,
              double *trace)
{
    cg_ws c;
    cg_init(&c, p);
    cgnr_ws(p, &c, (const cplx *)y, w, (cplx *)f_hat_iter, iters, trace);
    cg_free(&c);
}

/* Test hook: CGNR with every NFFT output multiplied by (1 + eps N(0,1)).
 * Measures how far the solver itself moves under operator errors of a
 * given size (the floor against which a reduced-precision solver is held). */
void orc_cgnr_perturbed(orc_nfft *p, const double *y, const double *w, double *f_hat_iter,
                        int iters, double eps, unsigned long seed)
{
    cg_ws c;
    cg_init(&c, p);
    c.noise = eps;
    c.rng = seed;
    cgnr_ws(p, &c, (const cplx *)y, w, (cplx *)f_hat_iter, iters, NULL);
    cg_free(&c);
}

/* ===================================================================== */
/* Denoising (src/denoise.c).  Volumes are flat [Z][Y][X]; the reference */
/* indexes them img[i][j][k] with i over its "nx" (= Z), j over "ny" (= Y)*/
/* and k over its "nz" (= X).  Loop order and arithmetic order follow it. */
/* ===================================================================== */

#define IDX(i, j, k) (((size_t)(i) * NY + (size_t)(j)) * NX + (size_t)(k))

static void tv_core(const double *img, double *out, float lam, int niter, int NZ, int NY,
                    int NX, int use_height, int nheight, int ncenter)
{
    /* denoise.c:67-151 (and the height variant, denoise.c:153-249) */
    size_t V = (size_t)NZ * NY * NX;
    double *u = out;
    double *grad = (double *)malloc(sizeof(double) * V);
    const double eps = 1e-8;
    memmove(u, img, sizeof(double) * V);
    int jlo = (2 * ncenter - nheight) / 2, jhi = (2 * ncenter + nheight) / 2;
    while (niter--) {
        double tmp0 = 0;
        /* The gradient of each voxel depends only on u, so it is computed in
         * parallel; the global sum below keeps the reference's (k, j, i)
         * order, so the result is bit-identical to the serial loops. */
#pragma omp parallel for schedule(static)
        for (int k = 0; k < NX; k++) {
            int kp = (k == NX - 1) ? NX - 1 : k + 1;
            int km = (k == 0) ? 0 : k - 1;
            for (int j = 0; j < NY; j++) {
                if (use_height && (j < jlo || j > jhi)) continue;
                int jp = (j == NY - 1) ? NY - 1 : j + 1;
                int jm = (j == 0) ? 0 : j - 1;
                for (int i = 0; i < NZ; i++) {
                    int ip = (i == NZ - 1) ? NZ - 1 : i + 1;
                    int im = (i == 0) ? 0 : i - 1;
                    double c = u[IDX(i, j, k)];
                    double t1 = c - u[IDX(im, j, k)];
                    double t2 = c - u[IDX(i, jm, k)];
                    double t3 = c - u[IDX(i, j, km)];
                    double a4 = u[IDX(ip, j, k)];
                    double t4 = a4 - c;
                    double t5 = a4 - u[IDX(ip, jm, k)];
                    double t6 = a4 - u[IDX(ip, j, km)];
                    double a7 = u[IDX(i, jp, k)];
                    double t7 = a7 - u[IDX(im, jp, k)];
                    double t8 = a7 - c;
                    double t9 = a7 - u[IDX(i, jp, km)];
                    double a10 = u[IDX(i, j, kp)];
                    double t10 = a10 - u[IDX(im, j, kp)];
                    double t11 = a10 - u[IDX(i, jm, kp)];
                    double t12 = a10 - c;
                    double g = (t1 + t2 + t3) / sqrt(eps + t1 * t1 + t2 * t2 + t3 * t3) -
                               t4 / sqrt(eps + t4 * t4 + t5 * t5 + t6 * t6) -
                               t8 / sqrt(eps + t7 * t7 + t8 * t8 + t9 * t9) -
                               t12 / sqrt(eps + t10 * t10 + t11 * t11 + t12 * t12);
                    grad[IDX(i, j, k)] = g;
                }
            }
        }
        for (int k = 0; k < NX; k++)
            for (int j = 0; j < NY; j++) {
                if (use_height && (j < jlo || j > jhi)) continue;
                for (int i = 0; i < NZ; i++) {
                    double g = grad[IDX(i, j, k)];
                    tmp0 += g * g;
                }
            }
        double dA = 0;
        double tn = sqrt(tmp0);
        for (int k = 0; k < NX; k++)
            for (int j = 0; j < NY; j++) {
                if (use_height && (j < jlo || j > jhi)) continue;
                for (int i = 0; i < NZ; i++) {
                    grad[IDX(i, j, k)] /= tn;
                    double c = u[IDX(i, j, k)];
                    if (c < 0) dA += c * c;
                }
            }
        double sa = sqrt(dA);
        for (int k = 0; k < NX; k++)
            for (int j = 0; j < NY; j++) {
                if (use_height && (j < jlo || j > jhi)) continue;
                for (int i = 0; i < NZ; i++) u[IDX(i, j, k)] -= lam * sa * grad[IDX(i, j, k)];
            }
    }
    free(grad);
}

void orc_tv_discrete(const double *img, double *out, float lam, int niter, int nz, int ny,
                     int nx)
{
    tv_core(img, out, lam, niter, nz, ny, nx, 0, 0, 0);
}

void orc_tv_discrete_height(const double *img, double *out, float lam, int niter, int nz,
                            int ny, int nx, int nheight, int ncenter)
{
    tv_core(img, out, lam, niter, nz, ny, nx, 1, nheight, ncenter);
}

/* denoise.c:320-378, in place (Gauss-Seidel) per Z-plane, rows then columns.
 * The reference compares the column index against its "nx" argument, which
 * the reconstruction passes as the number of Z-planes (reconstruction.c:627).
 * nx_bound carries that value.  Where the reference then reads one element
 * past the row (column NX), glibc allocator metadata sits there (0 or a
 * denormal below 1e-319); this restatement defines that value as 0.0. */
void orc_aniso_diffusion_2d(const double *img, double *out, float lambda, float kappa,
                            int niter, int NZ, int NY, int NX, int nx_bound)
{
    size_t V = (size_t)NZ * NY * NX;
    double *u = out;
    memmove(u, img, sizeof(double) * V);
    double Ksq = (double)kappa * (double)kappa;
    /* planes are independent: running them on several threads keeps every
     * plane's sequential Gauss-Seidel order and result */
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < NZ; k++) {
        for (int it = 0; it < niter; it++) {
            for (int j = 0; j < NY; j++) {
                int jp = (j == NY - 1) ? NY - 1 : j + 1;
                int jm = (j == 0) ? 0 : j - 1;
                for (int i = 0; i < NX; i++) {
                    int ip = (i == nx_bound - 1) ? nx_bound - 1 : i + 1;
                    int im = (i == 0) ? 0 : i - 1;
                    double c = u[IDX(k, j, i)];
                    double e = (ip < NX) ? u[IDX(k, j, ip)] : 0.0;
                    double gN = u[IDX(k, jm, i)] - c;
                    double gS = u[IDX(k, jp, i)] - c;
                    double gE = e - c;
                    double gW = u[IDX(k, j, im)] - c;
                    double cN = 1.0 / (1.0 + gN * gN / Ksq);
                    double cS = 1.0 / (1.0 + gS * gS / Ksq);
                    double cE = 1.0 / (1.0 + gE * gE / Ksq);
                    double cW = 1.0 / (1.0 + gW * gW / Ksq);
                    u[IDX(k, j, i)] = c + lambda * (cN * gN + cS * gS + cE * gE + cW * gW);
                }
            }
        }
    }
}

/* denoise.c:381-402 */
void orc_show_grad_mag(const double *img, double *out, int NZ, int NY, int NX)
{
    size_t V = (size_t)NZ * NY * NX;
    memmove(out, img, sizeof(double) * V);
    for (int i = 1; i < NZ - 1; i++)
        for (int j = 1; j < NY - 1; j++)
            for (int k = 1; k < NX - 1; k++) {
                double c = img[IDX(i, j, k)];
                double a = c - img[IDX(i - 1, j, k)];
                double b = c - img[IDX(i, j - 1, k)];
                double d = c - img[IDX(i, j, k - 1)];
                out[IDX(i, j, k)] = sqrt(a * a + b * b + d * d);
            }
}

/* ===================================================================== */
/* MT19937 (GSL default generator; seed 0 -> 4357)                        */
/* ===================================================================== */

void orc_mt19937_uniform(unsigned long seed, size_t n, double *out)
{
    uint32_t mt[624];
    int mti;
    uint32_t s = (uint32_t)(seed == 0 ? 4357 : seed);
    mt[0] = s;
    for (mti = 1; mti < 624; mti++)
        mt[mti] = (uint32_t)(1812433253UL * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti);
    for (size_t q = 0; q < n; q++) {
        if (mti >= 624) {
            for (int kk = 0; kk < 624; kk++) {
                uint32_t y = (mt[kk] & 0x80000000u) | (mt[(kk + 1) % 624] & 0x7fffffffu);
                mt[kk] = mt[(kk + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            mti = 0;
        }
        uint32_t y = mt[mti++];
        y ^= (y >> 11);
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= (y >> 18);
        out[q] = (double)y / 4294967296.0;
    }
}

/* ===================================================================== */
/* Full reconstruction                                                    */
/* ===================================================================== */

/* reconstruction.c:307-367: 2D NFFT of each tilt at uniform nodes. */
int orc_tilt_series_fourier(int nx, int nz, int np, int nslices, const double *proj,
                            double *tomograms_d)
{
    cplx *tomograms = (cplx *)tomograms_d;
    int M = np * nz;
    double *x = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    orc_uniform_sample_2d(np, nz, x);
    orc_nfft *p = orc_nfft_create(nx, nz, M, x);
    free(x);
    cplx *f_hat = (cplx *)malloc(sizeof(cplx) * (size_t)nx * nz);
    nfft_ws w;
    ws_init(&w, p);
    for (int j = 0; j < nslices; j++) {
        const double *pj = proj + (size_t)j * nx * nz;
        for (int i = 0; i < nx * nz; i++) {
            int col = i % nx, row = i / nx;
            f_hat[(size_t)col * nz + row] = pj[i];
        }
        nfft_trafo_ws(p, &w, f_hat, tomograms + (size_t)j * M);
    }
    ws_free(&w);
    free(f_hat);
    orc_nfft_destroy(p);
    return 0;
}

/* reconstruction.c:437-484: reorder, mask, fill. */
int orc_build_slices(const orc_recon_params *prm, const double *tomograms_d,
                     const double *fill, double *slices_d, int *mask)
{
    const cplx *tomograms = (const cplx *)tomograms_d;
    cplx *slices = (cplx *)slices_d;
    int np = prm->np, nz = prm->nz;
    double pad_min, pad_max;
    int A = orc_polar_lines(prm->gam_min, prm->gam_max, prm->interval, prm->padangle,
                            &pad_min, &pad_max);
    int ntotal1 = A * np, ntotal = np * nz;
    double *rnd = NULL;
    size_t nunk = 0, used = 0;
    if (prm->random && !fill) {
        /* count unknown entries, then draw that many in (z, i) order */
        for (int i = 0; i < ntotal1; i++) {
            int nslc = i / np;
            double angle = pad_min + nslc * prm->padangle;
            int span = (int)(prm->interval / prm->padangle + 0.5);
            int seq = (int)((angle - prm->gam_min) / prm->padangle + 0.5);
            if ((angle < prm->gam_min) || (angle > prm->gam_max) || (seq % span != 0) ||
                abs((int)angle) < 1e-5)
                nunk++;
        }
        nunk *= (size_t)nz;
        rnd = (double *)malloc(sizeof(double) * (nunk ? nunk : 1));
        orc_mt19937_uniform(0, nunk, rnd);
        for (size_t q = 0; q < nunk; q++) rnd[q] *= 10; /* gsl_rng_uniform(rng)*10 */
        fill = rnd;
    }
    for (int j = 0; j < nz; j++) {
        for (int i = 0; i < ntotal1; i++) {
            int nslc = i / np;
            double angle = pad_min + nslc * prm->padangle;
            int span = (int)(prm->interval / prm->padangle + 0.5);
            int seq = (int)((angle - prm->gam_min) / prm->padangle + 0.5);
            size_t o = (size_t)j * ntotal1 + i;
            if ((angle < prm->gam_min) || (angle > prm->gam_max) || (seq % span != 0) ||
                abs((int)angle) < 1e-5) {
                mask[o] = 0;
                slices[o] = prm->random ? fill[used++] : 0;
            } else {
                mask[o] = 1;
                int order = (int)((angle - prm->gam_min) / prm->interval + 0.5);
                int col = i % np;
                slices[o] = tomograms[(size_t)order * ntotal + (size_t)j * np + col];
            }
        }
    }
    free(rnd);
    return 0;
}

/* Staged form of reconstruction.c:304-719: begin = setup and initial
 * inverse (:304-540), iterate = outer HIO/ER iterations (:545-703). */
struct orc_recon {
    orc_recon_params prm;
    int M, nplanes, iters, nthreads, done;
    size_t PP, V;
    orc_nfft *pl;
    double *w;
    cplx *slices, *data;
    int *mask;
    double *img, *img_last, *den, *d1, *d2;
    double t_planes, t_volume;
};

static double wall(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

orc_recon *orc_recon_begin(const orc_recon_params *prm, const double *proj, const double *fill)
{
    int nx = prm->nx, nz = prm->nz, np = prm->np;
    if (nx <= 0 || nz <= 0 || np <= 0 || (nz & 1) || (np & 1)) return NULL;
    orc_recon *R = (orc_recon *)calloc(1, sizeof(orc_recon));
    R->prm = *prm;
    int nslices = (int)((prm->gam_max - prm->gam_min) / prm->interval + 0.5) + 1;
    R->iters = prm->cgnr_iters > 0 ? prm->cgnr_iters : 10;
    R->nthreads = prm->nthreads > 0 ? prm->nthreads : 1;
    R->nplanes = (prm->plane_limit > 0 && prm->plane_limit < nz) ? prm->plane_limit : nz;
    size_t PP = (size_t)np * np, V = PP * nz;
    R->PP = PP;
    R->V = V;
    int ntotal = np * nz;
    cplx *tomograms = (cplx *)malloc(sizeof(cplx) * (size_t)ntotal * nslices);
    orc_tilt_series_fourier(nx, nz, np, nslices, proj, (double *)tomograms);

    double pad_min, pad_max;
    int A = orc_polar_lines(prm->gam_min, prm->gam_max, prm->interval, prm->padangle,
                            &pad_min, &pad_max);
    int M = A * np;
    R->M = M;
    double *x = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    orc_equal_angle_sample_2d(pad_min, pad_max, prm->padangle, np, x);
    R->pl = orc_nfft_create(np, np, M, x);
    free(x);

    /* reconstruction.c:415-426 */
    if (prm->weight) {
        R->w = (double *)malloc(sizeof(double) * (size_t)M);
        for (int j = 0; j < A; j++)
            for (int i = 0; i < np; i++) {
                double h = (double)(np / 2);
                if (i == np / 2)
                    R->w[j * np + i] = REF_PI / (4 * A * (h * h));
                else
                    R->w[j * np + i] = prm->padangle / 180 * REF_PI * abs(i - np / 2) / (h * h);
            }
    }
    R->slices = (cplx *)malloc(sizeof(cplx) * (size_t)M * nz);
    R->mask = (int *)malloc(sizeof(int) * (size_t)M * nz);
    orc_build_slices(prm, (double *)tomograms, fill, (double *)R->slices, R->mask);
    free(tomograms);

    R->data = (cplx *)calloc(V, sizeof(cplx));
    R->img = (double *)malloc(sizeof(double) * V);
    R->img_last = (double *)malloc(sizeof(double) * V);
    R->den = (double *)malloc(sizeof(double) * V);
    R->d1 = (double *)malloc(sizeof(double) * nz);
    R->d2 = (double *)malloc(sizeof(double) * nz);

    /* reconstruction.c:495-518: initial inverse NFFT per plane */
    cplx *data = R->data;
#pragma omp parallel num_threads(R->nthreads)
    {
        cg_ws c;
        cg_init(&c, R->pl);
        cplx *f = (cplx *)malloc(sizeof(cplx) * PP);
#pragma omp for schedule(dynamic)
        for (int j = 0; j < R->nplanes; j++) {
            for (size_t i = 0; i < PP; i++) f[i] = 0.0;
            cgnr_ws(R->pl, &c, R->slices + (size_t)j * M, R->w, f, R->iters, NULL);
            for (size_t i = 0; i < PP; i++) data[((size_t)j * PP + i + V / 2) % V] = f[i];
        }
        free(f);
        cg_free(&c);
    }
    /* reconstruction.c:521-540 */
    orc_fft_many((double *)data, nz, (int)PP, (int)PP, 1, +1);
    for (int j = 0; j < nz; j++)
        for (size_t i = 0; i < PP; i++)
            R->img[(size_t)((j + nz / 2) % nz) * PP + i] = creal(data[(size_t)j * PP + i]) / nz;
    return R;
}

int orc_recon_iterate(orc_recon *R, int n, double *rhist_out)
{
    const orc_recon_params *prm = &R->prm;
    int nx = prm->nx, nz = prm->nz, np = prm->np, M = R->M;
    size_t PP = R->PP, V = R->V;
    cplx *data = R->data;
    double *img = R->img, *img_last = R->img_last;
    for (int q = 0; q < n && R->done < prm->nhio + prm->ner; q++) {
        int nn = R->done;
        double t0 = wall();
        /* :548-553 */
        for (int j = 0; j < nz; j++)
            for (size_t i = 0; i < PP; i++) {
                data[(size_t)j * PP + i] = img[(size_t)((j + nz / 2) % nz) * PP + i];
                img_last[(size_t)j * PP + i] = img[(size_t)j * PP + i];
            }
        /* :556-559 */
        orc_fft_many((double *)data, nz, (int)PP, (int)PP, 1, -1);
        double t1 = wall();
        /* :565-601 */
#pragma omp parallel num_threads(R->nthreads)
        {
            cg_ws c;
            cg_init(&c, R->pl);
            cplx *fh = (cplx *)malloc(sizeof(cplx) * PP);
            cplx *ff = (cplx *)malloc(sizeof(cplx) * (size_t)M);
            cplx *y = (cplx *)malloc(sizeof(cplx) * (size_t)M);
#pragma omp for schedule(dynamic)
            for (int j = 0; j < nz; j++) {
                R->d1[j] = 0;
                R->d2[j] = 0;
                if (j >= R->nplanes) continue;
                size_t base = ((size_t)j * PP + V / 2) % V;
                for (size_t i = 0; i < PP; i++) fh[i] = data[base + i];
                nfft_trafo_ws(R->pl, &c.nw, fh, ff);
                const cplx *s = R->slices + (size_t)j * M;
                const int *mk = R->mask + (size_t)j * M;
                double a1 = 0, a2 = 0;
                for (int i = 0; i < M; i++) {
                    if (mk[i] > 0.5) {
                        y[i] = s[i];
                        cplx dm = ff[i] - s[i], dp = ff[i] + s[i];
                        a1 += creal(dm) * creal(dm) + cimag(dm) * cimag(dm);
                        a2 += creal(dp) * creal(dp) + cimag(dp) * cimag(dp);
                    } else {
                        y[i] = ff[i];
                    }
                }
                R->d1[j] = a1;
                R->d2[j] = a2;
                const double *wp = img + (size_t)((j + nz / 2) % nz) * PP;
                for (size_t i = 0; i < PP; i++) fh[i] = wp[i];
                cgnr_ws(R->pl, &c, y, R->w, fh, R->iters, NULL);
                for (size_t i = 0; i < PP; i++) data[base + i] = fh[i];
            }
            free(fh);
            free(ff);
            free(y);
            cg_free(&c);
        }
        double t2 = wall();
        double diff1 = 0, diff2 = 0;
        for (int j = 0; j < nz; j++) {
            diff1 += R->d1[j];
            diff2 += R->d2[j];
        }
        if (rhist_out) rhist_out[nn] = sqrt(diff1 / diff2);
        /* :607-621 */
        orc_fft_many((double *)data, nz, (int)PP, (int)PP, 1, +1);
        for (size_t t = 0; t < V; t++) img[t] = creal(data[(t + V / 2) % V]) / nz;
        /* :624-669 (serial) / reconstruction-parallel.c:761-802 */
        if (prm->denoise == 2) {
            float lamd = prm->variant == 1 ? 0.4f : 0.25f;
            orc_aniso_diffusion_2d(img, R->den, lamd, 0.005f, 80, nz, np, np, nz);
            memcpy(img, R->den, sizeof(double) * V);
        } else if (prm->denoise == 1) {
            if (prm->height && prm->variant == 0)
                orc_tv_discrete_height(img, R->den, 0.2f, 40, nz, np, np, prm->nheight,
                                       prm->ncenter);
            else
                orc_tv_discrete(img, R->den, 0.2f, 40, nz, np, np);
            memcpy(img, R->den, sizeof(double) * V);
        }
        /* :672-700 (serial) / reconstruction-parallel.c:805-833 */
        int hio = nn < prm->nhio;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < nz; j++)
            for (size_t i = 0; i < PP; i++) {
                int yi = (int)(i / np), xi = (int)(i % np);
                size_t o = (size_t)j * PP + i;
                int inside;
                if (prm->height) {
                    if (prm->variant == 1)
                        inside = yi >= (np - prm->nheight) / 2 && yi <= (np + prm->nheight) / 2;
                    else
                        inside = yi >= (2 * prm->ncenter - prm->nheight) / 2 &&
                                 yi <= (2 * prm->ncenter + prm->nheight) / 2;
                } else {
                    inside = (yi >= (np - nx) / 2) && (yi < (np + nx) / 2) &&
                             (xi >= (np - nx) / 2) && (xi < (np + nx) / 2);
                }
                if (inside) {
                    if (img[o] < 0) img[o] = hio ? img_last[o] - 0.9 * img[o] : 0;
                } else {
                    img[o] = hio ? img_last[o] - 0.9 * img[o] : 0;
                }
            }
        double t3 = wall();
        R->t_planes += t2 - t1;
        R->t_volume += (t1 - t0) + (t3 - t2);
        R->done++;
    }
    return R->done;
}

void orc_recon_volume(const orc_recon *R, double *out)
{
    memcpy(out, R->img, sizeof(double) * R->V);
}

void orc_recon_times(const orc_recon *R, double *t_planes, double *t_volume)
{
    if (t_planes) *t_planes = R->t_planes;
    if (t_volume) *t_volume = R->t_volume;
}

void orc_recon_end(orc_recon *R)
{
    if (!R) return;
    orc_nfft_destroy(R->pl);
    free(R->w);
    free(R->slices);
    free(R->mask);
    free(R->data);
    free(R->img);
    free(R->img_last);
    free(R->den);
    free(R->d1);
    free(R->d2);
    free(R);
}

int orc_reconstruct(const orc_recon_params *prm, const double *proj, const double *fill,
                    double *vol0_out, double *vol_out, double *rhist_out)
{
    orc_recon *R = orc_recon_begin(prm, proj, fill);
    if (!R) return -1;
    if (vol0_out) orc_recon_volume(R, vol0_out);
    orc_recon_iterate(R, prm->nhio + prm->ner, rhist_out);
    if (vol_out) orc_recon_volume(R, vol_out);
    orc_recon_end(R);
    return 0;
}

/* ===================================================================== */
/* projection_sim -m 2D1D (src/projection_sim.c:282-405), without noise   */
/* ===================================================================== */

int orc_project_2d1d(const double *density, int nx, int ny, int nz, int np, double gam_min,
                     double gam_max, double interval, double *proj_out)
{
    int nslices = orc_equal_angle_count(gam_min, gam_max, interval);
    int M = nslices * np;
    double *x = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    orc_equal_angle_sample_2d(gam_min, gam_max, interval, np, x);
    orc_nfft *p = orc_nfft_create(ny, nx, M, x);
    free(x);
    size_t XY = (size_t)nx * ny, V = XY * nz;
    cplx *data = (cplx *)malloc(sizeof(cplx) * V);
    for (size_t t = 0; t < V; t++) data[t] = density[t];
    orc_fft_many((double *)data, nz, (int)XY, (int)XY, 1, -1);
    cplx *slices = (cplx *)malloc(sizeof(cplx) * (size_t)np * nz * nslices);
    cplx *fh = (cplx *)malloc(sizeof(cplx) * XY);
    cplx *f = (cplx *)malloc(sizeof(cplx) * (size_t)M);
    nfft_ws w;
    ws_init(&w, p);
    for (int j = 0; j < nz; j++) {
        for (size_t i = 0; i < XY; i++) fh[i] = data[((size_t)j * XY + i + V / 2) % V];
        nfft_trafo_ws(p, &w, fh, f);
        for (int i = 0; i < M; i++) {
            int nslc = i / np, ncol = i % np;
            slices[(size_t)nslc * np * nz + (size_t)j * np + ncol] = f[i];
        }
    }
    ws_free(&w);
    cplx *slice = (cplx *)malloc(sizeof(cplx) * (size_t)np * nz);
    fft_tw T0, T1;
    fft_tw_init(&T0, nz, +1);
    fft_tw_init(&T1, np, +1);
    int nm = nz > np ? nz : np;
    cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)nm);
    cplx *b = (cplx *)malloc(sizeof(cplx) * (size_t)nm);
    for (int j = 0; j < nslices; j++) {
        for (int i = 0; i < np * nz; i++) {
            int row = (i / np + nz / 2) % nz;
            int col = (i % np + np / 2) % np;
            slice[(size_t)row * np + col] = slices[(size_t)j * np * nz + i];
        }
        fft_2d(slice, nz, np, &T0, &T1, a, b);
        for (int i = 0; i < np * nz; i++) {
            int row = i / np, col = i % np, cs = (col + np / 2) % np;
            if (col >= np / 2) continue;
            cplx t = slice[(size_t)row * np + col];
            slice[(size_t)row * np + col] = slice[(size_t)row * np + cs];
            slice[(size_t)row * np + cs] = t;
        }
        for (int i = 0; i < np * nz; i++)
            proj_out[(size_t)j * np * nz + i] = creal(slice[i]) / (np * nz);
    }
    free(a);
    free(b);
    free(T0.tw);
    free(T1.tw);
    free(slice);
    free(slices);
    free(fh);
    free(f);
    free(data);
    orc_nfft_destroy(p);
    return 0;
}
