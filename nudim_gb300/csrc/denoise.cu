// denoise.cu -- TV-discrete (and its height-window variant) and the in-place
// 2D anisotropic diffusion of denoise.c, on [z][y][x] volumes.
//
// Arithmetic uses round-to-nearest intrinsics (no contraction) so that the
// FP64 form reproduces the reference's per-voxel C arithmetic exactly; only
// the two global sums of TV are summed in a different (tree) order.
#include "engine.cuh"

namespace nudim {

// ================================================================ TV
// denoise.c:67-151 / 153-249 called as total_variation_discrete(img, lam,
// niter, nz, np, np): the reference's i runs over Z, j over Y, k over X.
template <typename T>
__global__ void __launch_bounds__(256)
k_tv_grad(const T *__restrict__ u, T *__restrict__ g, double *__restrict__ part, int nz, int ny,
          int nx, int height, int ylo, int yhi)
{
    __shared__ double sh[32];
    size_t V = (size_t)nz * ny * nx;
    size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double sg = 0, sn = 0;
    if (o < V) {
        int k = (int)(o % nx);
        size_t q = o / nx;
        int j = (int)(q % ny);
        int i = (int)(q / ny);
        if (!height || (j >= ylo && j <= yhi)) {
            int ip = (i == nz - 1) ? nz - 1 : i + 1, im = (i == 0) ? 0 : i - 1;
            int jp = (j == ny - 1) ? ny - 1 : j + 1, jm = (j == 0) ? 0 : j - 1;
            int kp = (k == nx - 1) ? nx - 1 : k + 1, km = (k == 0) ? 0 : k - 1;
            auto at = [&](int a, int b, int c) { return u[((size_t)a * ny + b) * nx + c]; };
            const T eps = (T)1e-8;
            T c = u[o];
            T t1 = rn_sub(c, at(im, j, k));
            T t2 = rn_sub(c, at(i, jm, k));
            T t3 = rn_sub(c, at(i, j, km));
            T a4 = at(ip, j, k);
            T t4 = rn_sub(a4, c);
            T t5 = rn_sub(a4, at(ip, jm, k));
            T t6 = rn_sub(a4, at(ip, j, km));
            T a7 = at(i, jp, k);
            T t7 = rn_sub(a7, at(im, jp, k));
            T t8 = rn_sub(a7, c);
            T t9 = rn_sub(a7, at(i, jp, km));
            T a10 = at(i, j, kp);
            T t10 = rn_sub(a10, at(im, j, kp));
            T t11 = rn_sub(a10, at(i, jm, kp));
            T t12 = rn_sub(a10, c);
            auto nrm = [&](T x, T y, T z) {
                return rn_sqrt(rn_add(rn_add(rn_add(eps, rn_mul(x, x)), rn_mul(y, y)), rn_mul(z, z)));
            };
            T g1 = rn_div(rn_add(rn_add(t1, t2), t3), nrm(t1, t2, t3));
            T g2 = rn_div(t4, nrm(t4, t5, t6));
            T g3 = rn_div(t8, nrm(t7, t8, t9));
            T g4 = rn_div(t12, nrm(t10, t11, t12));
            T gv = rn_sub(rn_sub(rn_sub(g1, g2), g3), g4);
            g[o] = gv;
            sg = (double)gv * (double)gv;
            if (c < T(0)) sn = (double)c * (double)c;
        }
    }
    sg = block_sum(sg, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = sg;
    sn = block_sum(sn, sh);
    if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = sn;
}

// u -= (lam * sqrt(dA)) * (g / sqrt(sum g^2))   (denoise.c:125-142)
template <typename T>
__global__ void __launch_bounds__(256)
k_tv_update(T *__restrict__ u, const T *__restrict__ g, const double *__restrict__ scal,
            double lam, int nz, int ny, int nx, int height, int ylo, int yhi)
{
    size_t V = (size_t)nz * ny * nx;
    size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= V) return;
    if (height) {
        int j = (int)((o / nx) % ny);
        if (j < ylo || j > yhi) return;
    }
    T tn = (T)sqrt(scal[0]);
    T la = (T)(lam * sqrt(scal[1]));
    u[o] = rn_sub(u[o], rn_mul(la, rn_div(g[o], tn)));
}

int tv_part_count(int nz, int ny, int nx)
{
    return 2 * ceil_div((long)nz * ny * nx, 256) + 2;
}

template <typename T>
int tv_run(T *u, T *grad, double *part, int part_cap, double *scal, int nz, int ny, int nx,
           float lam, int niter, int height, int ylo, int yhi, cudaStream_t st)
{
    size_t V = (size_t)nz * ny * nx;
    int nb = ceil_div((long)V, 256);
    if (part_cap < 2 * nb) {
        set_error("tv_run: partial buffer too small");
        return NUDIM_EINVAL;
    }
    for (int it = 0; it < niter; it++) {
        k_tv_grad<T><<<nb, 256, 0, st>>>(u, grad, part, nz, ny, nx, height, ylo, yhi);
        NUDIM_LAUNCH_CHECK();
        launch_finish_sums(part, nb, 1, 2 * nb, scal, 2, 2, st);
        k_tv_update<T><<<nb, 256, 0, st>>>(u, grad, scal, (double)lam, nz, ny, nx, height, ylo,
                                           yhi);
        NUDIM_LAUNCH_CHECK();
    }
    return NUDIM_OK;
}

// ================================================================ diffusion
// denoise.c:320-378: per Z-plane, `niter` Gauss-Seidel sweeps in (y, x)
// order, updated in place.  Cell (y, x) of sweep s reads its N and W
// neighbours from sweep s and its S and E neighbours from sweep s-1, so the
// sweeps run as a pipelined anti-diagonal wavefront: at step t sweep s
// updates diagonal d = t - 2s.  The arithmetic of every cell is the
// reference's, so the result is bit-identical to the sequential loops.
template <typename T>
__global__ void __launch_bounds__(1024)
k_diffusion(T *u, int ny, int nx, int nxb, double lambda_d, double ksq_d, int niter)
{
    T *U = u + (size_t)blockIdx.x * ny * nx;
    const T lambda = (T)lambda_d, Ksq = (T)ksq_d, one = (T)1;
    int D = ny + nx - 1, L = min(ny, nx);
    int nsteps = D + 2 * (niter - 1);
    for (int t = 0; t < nsteps; t++) {
        int s_hi = min(niter - 1, t / 2);
        int a = t - (D - 1);
        int s_lo = a > 0 ? (a + 1) / 2 : 0;
        int nact = s_hi - s_lo + 1;
        for (int w = threadIdx.x; w < nact * L; w += blockDim.x) {
            int s = s_lo + w / L, c = w - (w / L) * L;
            int d = t - 2 * s;
            int y0 = max(0, d - (nx - 1)), y1 = min(ny - 1, d);
            int y = y0 + c;
            if (y > y1) continue;
            int x = d - y;
            int jp = (y == ny - 1) ? ny - 1 : y + 1, jm = (y == 0) ? 0 : y - 1;
            int ip = (x == nxb - 1) ? nxb - 1 : x + 1, im = (x == 0) ? 0 : x - 1;
            T cv = U[(size_t)y * nx + x];
            T e = ip < nx ? U[(size_t)y * nx + ip] : T(0);
            T gN = rn_sub(U[(size_t)jm * nx + x], cv);
            T gS = rn_sub(U[(size_t)jp * nx + x], cv);
            T gE = rn_sub(e, cv);
            T gW = rn_sub(U[(size_t)y * nx + im], cv);
            T cN = rn_div(one, rn_add(one, rn_div(rn_mul(gN, gN), Ksq)));
            T cS = rn_div(one, rn_add(one, rn_div(rn_mul(gS, gS), Ksq)));
            T cE = rn_div(one, rn_add(one, rn_div(rn_mul(gE, gE), Ksq)));
            T cW = rn_div(one, rn_add(one, rn_div(rn_mul(gW, gW), Ksq)));
            T sum = rn_add(rn_add(rn_add(rn_mul(cN, gN), rn_mul(cS, gS)), rn_mul(cE, gE)),
                           rn_mul(cW, gW));
            U[(size_t)y * nx + x] = rn_add(cv, rn_mul(lambda, sum));
        }
        __syncthreads();
    }
}

template <typename T>
int diffusion_run(T *u, int nz, int ny, int nx, int nx_bound, float lambda, float kappa,
                  int niter, cudaStream_t st)
{
    if (niter <= 0 || nz <= 0) return NUDIM_OK;
    double ksq = (double)kappa * (double)kappa;
    k_diffusion<T><<<nz, 1024, 0, st>>>(u, ny, nx, nx_bound, (double)lambda, ksq, niter);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

template int tv_run<double>(double *, double *, double *, int, double *, int, int, int, float,
                            int, int, int, int, cudaStream_t);
template int tv_run<float>(float *, float *, double *, int, double *, int, int, int, float, int,
                           int, int, int, cudaStream_t);
template int diffusion_run<double>(double *, int, int, int, int, float, float, int, cudaStream_t);
template int diffusion_run<float>(float *, int, int, int, int, float, float, int, cudaStream_t);

}  // namespace nudim
