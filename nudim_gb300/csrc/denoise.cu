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
// One cell of denoise.c:320-378.  FP64: the reference's 1 / (1 + g^2 / K^2)
// with IEEE operations in its order (bit-identical).  FP32 form: the same
// coefficient as K^2 / (K^2 + g^2) with a fast division (relative error a few
// ulp per cell).
__device__ __forceinline__ double diff_coef(double g, double Ksq)
{
    return rn_div(1.0, rn_add(1.0, rn_div(rn_mul(g, g), Ksq)));
}
__device__ __forceinline__ float diff_coef(float g, float Ksq)
{
    return __fdividef(Ksq, Ksq + g * g);
}

template <typename T>
__device__ __forceinline__ T diff_cell(T cv, T nN, T nS, T nE, T nW, T lambda, T Ksq)
{
    T gN = rn_sub(nN, cv), gS = rn_sub(nS, cv), gE = rn_sub(nE, cv), gW = rn_sub(nW, cv);
    T cN = diff_coef(gN, Ksq), cS = diff_coef(gS, Ksq), cE = diff_coef(gE, Ksq),
      cW = diff_coef(gW, Ksq);
    T sum = rn_add(rn_add(rn_add(rn_mul(cN, gN), rn_mul(cS, gS)), rn_mul(cE, gE)),
                   rn_mul(cW, gW));
    return rn_add(cv, rn_mul(lambda, sum));
}

// Per Z-plane, `niter` Gauss-Seidel sweeps in (y, x) order, updated in
// place.  Cell (y, x) of sweep s reads its N and W neighbours from sweep s
// and its S and E neighbours from sweep s-1, so the sweeps run as a
// pipelined anti-diagonal wavefront: at step t sweep s updates diagonal
// d = t - 2s.  Every cell sees the neighbour values of the sequential loops.
// This form works in global memory (any plane size).
template <typename T>
__global__ void __launch_bounds__(1024)
k_diffusion(T *u, int ny, int nx, int nxb, double lambda_d, double ksq_d, int niter)
{
    T *U = u + (size_t)blockIdx.x * ny * nx;
    const T lambda = (T)lambda_d, Ksq = (T)ksq_d;
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
            U[(size_t)y * nx + x] = diff_cell<T>(cv, U[(size_t)jm * nx + x],
                                                 U[(size_t)jp * nx + x], e,
                                                 U[(size_t)y * nx + im], lambda, Ksq);
        }
        __syncthreads();
    }
}

// The same wavefront with the live band in shared memory.  Sweeps run in
// groups of G; inside a group sweep g updates anti-diagonal d = t - 2g at
// step t, so only diagonals [t - 2G + 1, t + 1] are live: they sit in a ring
// of R = 2G + 2 diagonal slots (slot = d mod R, cell (y, x) of diagonal d at
// position y - y0(d)).  During step t diagonal t + 2 is fetched into
// registers (its slot held diagonal t + 2 - R, written back at step t - 1)
// and diagonal t - 2G + 1, final for the group, is written back: one barrier
// per step.  Requires min(ny, nx) <= kDiffPf * blockDim.x.
constexpr int kDiffPf = 4;

template <typename T>
__global__ void __launch_bounds__(1024)
k_diffusion_ring(T *u, int ny, int nx, int nxb, double lambda_d, double ksq_d, int niter,
                 int G, int R)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T *ring = (T *)smraw;
    T *U = u + (size_t)blockIdx.x * ny * nx;
    const T lambda = (T)lambda_d, Ksq = (T)ksq_d;
    const int D = ny + nx - 1, L = min(ny, nx);
    const int P = min((int)blockDim.x, (L + 31) & ~31), gs = blockDim.x / P;
    const int gi = threadIdx.x / P, i0 = threadIdx.x - gi * P;
    auto y0 = [&](int d) { return max(0, d - (nx - 1)); };
    auto len = [&](int d) { return min(d, ny - 1) - y0(d) + 1; };
    auto slot = [&](int d) { return ring + (size_t)(d % R) * L; };
    auto cell = [&](int d, int i) -> size_t {
        int a = y0(d);
        return (size_t)(a + i) * nx + (d - a - i);
    };
    for (int s0 = 0; s0 < niter; s0 += G) {
        const int gc = min(G, niter - s0);
        const int nsteps = D + 2 * (gc - 1);
        for (int d = 0; d < 2 && d < D; d++) {
            T *s = slot(d);
            for (int i = threadIdx.x; i < len(d); i += blockDim.x) s[i] = U[cell(d, i)];
        }
        __syncthreads();
        for (int t = 0; t < nsteps; t++) {
            // fetch diagonal t + 2
            const int dn = t + 2;
            const int nn = dn < D ? len(dn) : 0;
            T pf[kDiffPf];
#pragma unroll
            for (int k = 0; k < kDiffPf; k++) {
                int i = threadIdx.x + k * blockDim.x;
                pf[k] = i < nn ? U[cell(dn, i)] : T(0);
            }
            int g_hi = min(gc - 1, t / 2);
            int a = t - (D - 1);
            int g_lo = a > 0 ? (a + 1) / 2 : 0;
            // P threads per diagonal, gs diagonals at a time; the ring slot of
            // diagonal d = t - 2g moves down by 2 gs per g (no division)
            if (gi < gs && g_lo + gi <= g_hi) {
                int sd = (t - 2 * (g_lo + gi)) % R;
                for (int g = g_lo + gi; g <= g_hi; g += gs) {
                    const int d = t - 2 * g;
                    const int yd = y0(d), nd = min(d, ny - 1) - yd + 1;
                    if (i0 < nd) {
                        T *sc = ring + (size_t)sd * L;
                        const T *sm = d > 0 ? ring + (size_t)(sd == 0 ? R - 1 : sd - 1) * L : sc;
                        const T *sp = ring + (size_t)(sd == R - 1 ? 0 : sd + 1) * L;
                        const int ym = y0(d > 0 ? d - 1 : d), yp = y0(d + 1);
                        for (int i = i0; i < nd; i += P) {
                            int y = yd + i, x = d - y;
                            T cv = sc[i];
                            T nN = cv, nS = cv, nW = cv, nE = cv;
                            if (y > 0) nN = sm[(y - 1) - ym];
                            if (x > 0) nW = sm[y - ym];
                            if (y < ny - 1) nS = sp[(y + 1) - yp];
                            int ip = (x == nxb - 1) ? nxb - 1 : x + 1;
                            if (ip != x) nE = ip < nx ? sp[y - yp] : T(0);
                            sc[i] = diff_cell<T>(cv, nN, nS, nE, nW, lambda, Ksq);
                        }
                    }
                    sd -= 2 * gs;
                    if (sd < 0) sd += R;
                }
            }
            if (nn > 0) {
                T *s = slot(dn);
#pragma unroll
                for (int k = 0; k < kDiffPf; k++) {
                    int i = threadIdx.x + k * blockDim.x;
                    if (i < nn) s[i] = pf[k];
                }
            }
            const int df = t - 2 * gc + 1;  // final for this group
            if (df >= 0 && df < D) {
                const T *s = slot(df);
                for (int i = threadIdx.x; i < len(df); i += blockDim.x) U[cell(df, i)] = s[i];
            }
            __syncthreads();
        }
        {
            const T *s = slot(D - 1);
            for (int i = threadIdx.x; i < len(D - 1); i += blockDim.x) U[cell(D - 1, i)] = s[i];
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
    int L = ny < nx ? ny : nx;
    int P = std::min(1024, (L + 31) & ~31);
    // FP32 on planes up to 512 wide: two diagonals at a time, two CTAs per
    // SM; otherwise one CTA of 1024 threads with up to 160 KB of ring
    bool two = sizeof(T) == 4 && P <= 512;
    int threads = two ? 2 * P : 1024;
    const size_t budget = two ? ((size_t)110 << 10) : ((size_t)160 << 10);
    int G = (int)((budget / (sizeof(T) * (size_t)L) - 2) / 2);
    if (G > niter) G = niter;
    if (G >= 1 && L <= kDiffPf * threads) {
        int R = 2 * G + 2;
        size_t smem = sizeof(T) * (size_t)R * L;
        NUDIM_CUDA(cudaFuncSetAttribute(k_diffusion_ring<T>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        160 << 10));
        k_diffusion_ring<T><<<nz, threads, smem, st>>>(u, ny, nx, nx_bound, (double)lambda, ksq,
                                                        niter, G, R);
    } else {
        k_diffusion<T><<<nz, 1024, 0, st>>>(u, ny, nx, nx_bound, (double)lambda, ksq, niter);
    }
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
