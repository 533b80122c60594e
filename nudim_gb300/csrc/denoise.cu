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
    if (sizeof(T) == 4) {
        // FP32 form: the same sum with fused multiply-adds
        T sum = cN * gN;
        sum = fma(cS, gS, sum);
        sum = fma(cE, gE, sum);
        sum = fma(cW, gW, sum);
        return fma(lambda, sum, cv);
    }
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
// per step.  The cells of a step are dealt out as 64-cell segments of the
// active diagonals, one warp per segment, from a task table (segment prefix
// counts and ring slots) that warp 0 builds for step t + 1 during step t.
// Requires min(ny, nx) <= kDiffPf * blockDim.x.
constexpr int kDiffPf = 4;
constexpr int kDiffMaxG = 64;  // sweeps per group (task tables in shared memory)

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
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    // per step (double-buffered), for active diagonal k (sweep g_lo + k):
    // prefix count of its 64-cell tasks, d, y0(d), len(d), and the ring offsets
    // of diagonals d, d - 1, d + 1
    constexpr int TC = 64;
    __shared__ int s_pre[2][kDiffMaxG + 1], s_meta[2][2];
    __shared__ int4 s_dg[2][kDiffMaxG];   // d, y0, len, ring offset of d
    __shared__ int2 s_nb[2][kDiffMaxG];   // ring offsets of d - 1 (d itself when d == 0) and d + 1
    auto y0 = [&](int d) { return max(0, d - (nx - 1)); };
    auto len = [&](int d) { return min(d, ny - 1) - y0(d) + 1; };
    // warp 0: the task table of step t of a group of gc sweeps into buffer b
    auto build_table = [&](int t, int gc, int b) {
        const int g_hi = min(gc - 1, t / 2), a = t - (D - 1);
        const int g_lo = a > 0 ? (a + 1) / 2 : 0, nact = g_hi - g_lo + 1;
        int carry = 0;
        for (int base = 0; base < nact; base += 32) {
            const int k = base + lane;
            int c = 0;
            if (k < nact) {
                const int d = t - 2 * (g_lo + k), nd = len(d), sd = d % R;
                c = (nd + TC - 1) / TC;
                s_dg[b][k] = make_int4(d, y0(d), nd, sd * L);
                s_nb[b][k] = make_int2(d > 0 ? (sd == 0 ? R - 1 : sd - 1) * L : sd * L,
                                       (sd == R - 1 ? 0 : sd + 1) * L);
            }
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (k < nact) s_pre[b][k + 1] = carry + incl;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) {
            s_pre[b][0] = 0;
            s_meta[b][0] = nact;
            s_meta[b][1] = g_lo;
        }
    };
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
        if (warp == 0) build_table(0, gc, 0);
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
            // the next step's task table (warp 0), then this step's tasks:
            // 64-cell segments of the active diagonals, dealt out to the warps
            const int tb = t & 1;
            if (warp == 0 && t + 1 < nsteps) build_table(t + 1, gc, tb ^ 1);
            {
                const int *pre = s_pre[tb];
                const int nact = s_meta[tb][0], ntask = pre[nact];
                // this warp's contiguous share of the tasks; k: the diagonal of
                // the first one (binary search over the prefix counts)
                const int t_beg = (int)((long)ntask * warp / nwarps);
                const int t_end = (int)((long)ntask * (warp + 1) / nwarps);
                int k = 0;
                for (int lo = 0, hi = nact - 1; lo <= hi;) {
                    int mid = (lo + hi) >> 1;
                    if (pre[mid + 1] <= t_beg) lo = mid + 1, k = lo;
                    else hi = mid - 1;
                }
                for (int task = t_beg; task < t_end; task++) {
                    while (pre[k + 1] <= task) k++;
                    const int4 dg = s_dg[tb][k];
                    const int2 nb = s_nb[tb][k];
                    const int d = dg.x, yd = dg.y, nd = dg.z;
                    // rows of diagonal d's neighbours: y0(d - 1) and y0(d + 1)
                    const int ym = d > nx - 1 ? yd - 1 : 0, yp = d + 1 > nx - 1 ? yd + 1 : 0;
                    T *sc = ring + dg.w;
                    const T *sm = ring + nb.x, *sp = ring + nb.y;
                    const int i0 = (task - pre[k]) * TC;
                    const T *mb = sm + (yd - ym), *pb = sp + (yd - yp);
#pragma unroll
                    for (int h = 0; h < TC / 32; h++) {
                        const int g0 = i0 + h * 32, g1 = min(nd, g0 + 32) - 1, i = g0 + lane;
                        // an interior group of 32 cells: each has its four plain
                        // neighbours (y in [1, ny-2], x in [1, nx-2] and x != nxb - 1,
                        // the column the reference clamps): cell i's N and W sit at
                        // i - 1, i of diagonal d - 1 from yd - ym, its S and E at i + 1,
                        // i of diagonal d + 1 from yd - yp.  Along a diagonal y grows
                        // and x falls.
                        const int xmax = d - yd - g0, xmin = d - yd - g1;
                        const bool inner = g0 <= g1 && yd + g0 >= 1 && yd + g1 <= ny - 2 &&
                                           xmin >= 1 && xmax <= nx - 2 &&
                                           !(xmin <= nxb - 1 && nxb - 1 <= xmax);
                        if (__all_sync(0xffffffffu, inner)) {  // warp-uniform: a real branch
                            if (i <= g1) {
                                T cv = sc[i];
                                sc[i] = diff_cell<T>(cv, mb[i - 1], pb[i + 1], pb[i], mb[i], lambda,
                                                     Ksq);
                            }
                        } else if (i <= g1) {
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
    const size_t budget = two ? ((size_t)108 << 10) : ((size_t)160 << 10);
    int G = (int)((budget / (sizeof(T) * (size_t)L) - 2) / 2);
    if (G > niter) G = niter;
    if (G > kDiffMaxG) G = kDiffMaxG;
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
