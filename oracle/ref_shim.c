/*
 * ref_shim.c -- flat-array adapters around the reference's own denoise.c and
 * grid.c (compiled from the reference tree by `make ref`).  Test
 * infrastructure: it exists only to generate golden vectors that pin the
 * oracle restatement (tests/golden/make_golden.py).
 *
 * The reference keeps volumes as double*** img[i][j][k] built by
 * malloc_image (denoise.c:404-421); these adapters copy a flat [i][j][k]
 * array in and out of that layout and call the reference functions unchanged.
 */
#include "grid.h"
#include "denoise.h"

static double ***to3(const double *a, int n0, int n1, int n2)
{
    double ***im = malloc_image(n0, n1, n2);
    for (int i = 0; i < n0; i++)
        for (int j = 0; j < n1; j++)
            memcpy(im[i][j], a + ((size_t)i * n1 + j) * n2, sizeof(double) * n2);
    return im;
}

static void from3(double ***im, double *a, int n0, int n1, int n2)
{
    for (int i = 0; i < n0; i++)
        for (int j = 0; j < n1; j++)
            memcpy(a + ((size_t)i * n1 + j) * n2, im[i][j], sizeof(double) * n2);
}

/* denoise.c:67-151 called as total_variation_discrete(img, lam, niter, n0, n1, n2) */
void ref_tv(const double *img, double *out, float lam, int niter, int n0, int n1, int n2)
{
    double ***a = to3(img, n0, n1, n2);
    double ***d = total_variation_discrete(a, lam, niter, n0, n1, n2);
    from3(d, out, n0, n1, n2);
    free_image(a, n0, n1);
    free_image(d, n0, n1);
}

/* denoise.c:153-249 */
void ref_tv_height(const double *img, double *out, float lam, int niter, int n0, int n1,
                   int n2, int nheight, int ncenter)
{
    double ***a = to3(img, n0, n1, n2);
    double ***d = total_variation_discrete_height(a, lam, niter, n0, n1, n2, nheight, ncenter);
    from3(d, out, n0, n1, n2);
    free_image(a, n0, n1);
    free_image(d, n0, n1);
}

/* denoise.c:320-378 */
void ref_diffusion_2d(const double *img, double *out, float lambda, float kappa, int niter,
                      int n0, int n1, int n2)
{
    double ***a = to3(img, n0, n1, n2);
    double ***d = aniso_diffusion_2d(a, lambda, kappa, niter, n0, n1, n2);
    from3(d, out, n0, n1, n2);
    free_image(a, n0, n1);
    free_image(d, n0, n1);
}

/* denoise.c:381-402 */
void ref_grad_mag(const double *img, double *out, int n0, int n1, int n2)
{
    double ***a = to3(img, n0, n1, n2);
    double ***d = show_grad_mag(a, n0, n1, n2);
    from3(d, out, n0, n1, n2);
    free_image(a, n0, n1);
    free_image(d, n0, n1);
}

/* grid.c:78-97 and 100-133, copied into caller buffers. */
int ref_equal_angle_sample_2D(double amin, double amax, double ai, int nx, double *out)
{
    int nt;
    double *x = equal_angle_sample_2D(amin, amax, ai, nx, &nt);
    memcpy(out, x, sizeof(double) * 2 * (size_t)nt);
    free(x);
    return nt;
}

int ref_uniform_sample_2D(int nx, int nz, double *out)
{
    int nt;
    double *x = uniform_sample_2D(nx, nz, &nt);
    memcpy(out, x, sizeof(double) * 2 * (size_t)nt);
    free(x);
    return nt;
}
