// ops.cu -- CGNR vector algebra, Z-axis pack/unpack, HIO/ER constraints,
// R-factor finish and the setup kernels (tilt-series transpose, slice
// reorder/mask/fill).
#include "engine.cuh"

namespace nudim {

// ================================================================ CGNR
// dots[p*4 + 0/1]: |z|^2 ping-pong, dots[p*4 + 2]: v^H W v.
template <typename T>
__global__ void __launch_bounds__(256)
k_cg_update(cplx_t<T> *__restrict__ f, const cplx_t<T> *__restrict__ p, cplx_t<T> *__restrict__ r,
            const cplx_t<T> *__restrict__ v, const double *__restrict__ dots, int cur, int N,
            int M)
{
    // one FP64 division per block (FP64 is slow here), shared with the block
    __shared__ T s_alpha;
    int b = blockIdx.y;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (threadIdx.x == 0) s_alpha = (T)(dots[b * 4 + cur] / dots[b * 4 + 2]);
    __syncthreads();
    const T alpha = s_alpha;
    if (i < (size_t)N) {
        size_t o = (size_t)b * N + i;
        cplx_t<T> fv = f[o], pv = p[o];
        fv.x += alpha * pv.x;
        fv.y += alpha * pv.y;
        f[o] = fv;
    } else if (i < (size_t)N + M) {
        size_t o = (size_t)b * M + (i - N);
        cplx_t<T> rv = r[o], vv = v[o];
        rv.x -= alpha * vv.x;
        rv.y -= alpha * vv.y;
        r[o] = rv;
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_cg_pupdate(cplx_t<T> *__restrict__ p, const cplx_t<T> *__restrict__ z,
             const double *__restrict__ dots, int cur, int nxt, int N)
{
    __shared__ T s_beta;
    int b = blockIdx.y;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (threadIdx.x == 0) s_beta = (T)(dots[b * 4 + nxt] / dots[b * 4 + cur]);
    __syncthreads();
    if (i >= (size_t)N) return;
    const T beta = s_beta;
    size_t o = (size_t)b * N + i;
    cplx_t<T> pv = p[o], zv = z[o];
    p[o] = mkc<T>(beta * pv.x + zv.x, beta * pv.y + zv.y);
}

// The coefficient-space step of the Toeplitz form: alpha = |z|^2 / p^H T p;
// f += alpha p; z -= alpha q (q = T p); per-block partial of |z'|^2.
template <typename T>
__global__ void __launch_bounds__(256)
k_cgt_update(cplx_t<T> *__restrict__ f, const cplx_t<T> *__restrict__ p, cplx_t<T> *__restrict__ z,
             const cplx_t<T> *__restrict__ q, const double *__restrict__ dots, int cur, int N,
             double *__restrict__ part, int part_stride)
{
    __shared__ T s_alpha;
    __shared__ double sh[32];
    const int b = blockIdx.y;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (threadIdx.x == 0) s_alpha = (T)(dots[b * 4 + cur] / dots[b * 4 + 2]);
    __syncthreads();
    const T alpha = s_alpha;
    T s = 0;
    if (i < (size_t)N) {
        const size_t o = (size_t)b * N + i;
        cplx_t<T> fv = f[o], zv = z[o];
        const cplx_t<T> pv = p[o], qv = q[o];
        fv.x += alpha * pv.x;
        fv.y += alpha * pv.y;
        zv.x -= alpha * qv.x;
        zv.y -= alpha * qv.y;
        f[o] = fv;
        z[o] = zv;
        s = zv.x * zv.x + zv.y * zv.y;
    }
    const double d = block_sum_t<T>(s, sh);
    if (threadIdx.x == 0) part[(size_t)b * part_stride + blockIdx.x] = d;
}

// CGNR with the normal operator T = A^H W A applied by Toeplitz embedding:
// z0 = A^H W y - T f0 (one adjoint NFFT), then per step q = T p with p^H q
// (= v^H W v for v = A p), f += alpha p, z -= alpha q (= A^H W r after
// r -= alpha v), p = z + beta p: the iterates of cgnr_run's NFFT form in
// exact arithmetic, one operator pass per step instead of a trafo and an
// adjoint.
template <typename T>
static int cgnr_run_toeplitz(NfftDev<T> &pl, int nplanes, const cplx_t<T> *y, const T *w,
                             cplx_t<T> *f, const T *f_real, bool f_zero, int iters,
                             CgnrBuffers<T> &b, cudaStream_t st)
{
    using C = cplx_t<T>;
    const int N = pl.N0 * pl.N1;
    SpreadArgs<T> sa;
    sa.f = y;
    sa.f_stride = pl.M;
    sa.w = w;
    if (f_zero) {
        NUDIM_CUDA(cudaMemsetAsync(f, 0, sizeof(C) * (size_t)N * nplanes, st));
        CropArgs<T> ca;
        ca.mode = CM_INIT;
        ca.out = b.z;
        ca.out_stride = N;
        ca.p_out = b.p;
        ca.part = b.part;
        ca.part_stride = b.part_stride;
        NUDIM_TRY(pl.adjoint(nplanes, sa, ca, st));
    } else {
        CropArgs<T> ca;
        ca.mode = CM_PLAIN;
        ca.out = b.z;
        ca.out_stride = N;
        NUDIM_TRY(pl.adjoint(nplanes, sa, ca, st));
        PadArgs<T> pa;
        if (f_real) {
            pa.mode = PM_REAL_INIT;
            pa.src = f_real;
            pa.f_init = f;
            pa.f_stride = N;
        } else {
            pa.src = f;
        }
        pa.src_stride = N;
        CropArgs<T> cr;
        cr.mode = CM_TRESID;
        cr.out = b.z;
        cr.out_stride = N;
        cr.p_out = b.p;
        cr.part = b.part;
        cr.part_stride = b.part_stride;
        NUDIM_TRY(pl.toeplitz_apply(nplanes, pa, cr, st));
    }
    launch_finish_sums(b.part, pl.crop_blocks(), nplanes, b.part_stride, b.dots + 0, 4, 1, st);
    NUDIM_LAUNCH_CHECK();
    int cur = 0;
    for (int it = 0; it < iters; it++) {
        PadArgs<T> pa;
        pa.src = b.p;
        pa.src_stride = N;
        CropArgs<T> cq;
        cq.mode = CM_TPDOT;
        cq.out = b.q;
        cq.out_stride = N;
        cq.pin = b.p;
        cq.part = b.part;
        cq.part_stride = b.part_stride;
        NUDIM_TRY(pl.toeplitz_apply(nplanes, pa, cq, st));
        launch_finish_sums(b.part, pl.crop_blocks(), nplanes, b.part_stride, b.dots + 2, 4, 1, st);
        const int nxt = 1 - cur;
        {
            ProfScope ps(pl.ctx, PK_CGVEC, st, 6.0 * sizeof(C) * (double)N * nplanes);
            dim3 gu(ceil_div(N, 256), nplanes);
            k_cgt_update<T><<<gu, 256, 0, st>>>(f, b.p, b.z, b.q, b.dots, cur, N, b.part,
                                                b.part_stride);
            NUDIM_LAUNCH_CHECK();
            launch_finish_sums(b.part, ceil_div(N, 256), nplanes, b.part_stride, b.dots + nxt, 4,
                               1, st);
        }
        {
            ProfScope ps(pl.ctx, PK_CGVEC, st, 3.0 * sizeof(C) * (double)N * nplanes);
            dim3 gp(ceil_div(N, 256), nplanes);
            k_cg_pupdate<T><<<gp, 256, 0, st>>>(b.p, b.z, b.dots, cur, nxt, N);
            NUDIM_LAUNCH_CHECK();
        }
        cur = nxt;
    }
    return NUDIM_OK;
}

int cgnr_part_stride(int M, int N)
{
    int a = 2 * ceil_div(M, 256), b = ceil_div(N, 256);
    return a > b ? a : b;
}

template <typename T>
int cgnr_run(NfftDev<T> &pl, int nplanes, const cplx_t<T> *y, const T *w, cplx_t<T> *f,
             const T *f_real, bool f_zero, int iters, CgnrBuffers<T> &b, cudaStream_t st)
{
    using C = cplx_t<T>;
    if (b.q && pl.toeplitz)
        return cgnr_run_toeplitz<T>(pl, nplanes, y, w, f, f_real, f_zero, iters, b, st);
    int N = pl.N0 * pl.N1, M = pl.M;
    // ---- solver_before_loop: r = y - A f; z = A^H W r; p = z
    if (f_real) {
        PadArgs<T> pa;
        pa.mode = PM_REAL_INIT;
        pa.src = f_real;
        pa.src_stride = N;
        pa.f_init = f;
        pa.f_stride = N;
        InterpArgs<T> ia;
        ia.mode = IM_RESID;
        ia.out = b.r;
        ia.out_stride = M;
        ia.y = y;
        ia.y_stride = M;
        NUDIM_TRY(pl.trafo(nplanes, pa, ia, st));
    } else if (f_zero) {
        NUDIM_CUDA(cudaMemsetAsync(f, 0, sizeof(C) * (size_t)N * nplanes, st));
        NUDIM_CUDA(cudaMemcpyAsync(b.r, y, sizeof(C) * (size_t)M * nplanes,
                                   cudaMemcpyDeviceToDevice, st));
    } else {
        PadArgs<T> pa;
        pa.src = f;
        pa.src_stride = N;
        InterpArgs<T> ia;
        ia.mode = IM_RESID;
        ia.out = b.r;
        ia.out_stride = M;
        ia.y = y;
        ia.y_stride = M;
        NUDIM_TRY(pl.trafo(nplanes, pa, ia, st));
    }
    SpreadArgs<T> sa;
    sa.f = b.r;
    sa.f_stride = M;
    sa.w = w;
    CropArgs<T> ca;
    ca.mode = CM_INIT;
    ca.out = b.z;
    ca.out_stride = N;
    ca.p_out = b.p;
    ca.part = b.part;
    ca.part_stride = b.part_stride;
    NUDIM_TRY(pl.adjoint(nplanes, sa, ca, st));
    launch_finish_sums(b.part, pl.crop_blocks(), nplanes, b.part_stride, b.dots + 0, 4, 1, st);
    NUDIM_LAUNCH_CHECK();
    int cur = 0;
    for (int it = 0; it < iters; it++) {
        // v = A p, dot_v = v^H W v
        PadArgs<T> pa;
        pa.src = b.p;
        pa.src_stride = N;
        InterpArgs<T> ia;
        ia.mode = IM_DOTV;
        ia.out = b.v;
        ia.out_stride = M;
        ia.w = w;
        ia.part = b.part;
        ia.part_stride = b.part_stride;
        NUDIM_TRY(pl.trafo(nplanes, pa, ia, st));
        launch_finish_sums(b.part, pl.interp_blocks(), nplanes, b.part_stride, b.dots + 2, 4, 1,
                           st);
        // alpha = |z|^2 / dot_v; f += alpha p; r -= alpha v
        {
            ProfScope ps(pl.ctx, PK_CGVEC, st, 3.0 * sizeof(C) * ((double)N + M) * nplanes);
            dim3 gu(ceil_div((long)N + M, 256), nplanes);
            k_cg_update<T><<<gu, 256, 0, st>>>(f, b.p, b.r, b.v, b.dots, cur, N, M);
            NUDIM_LAUNCH_CHECK();
        }
        // z = A^H W r, |z|^2
        CropArgs<T> cz;
        cz.mode = CM_DOT;
        cz.out = b.z;
        cz.out_stride = N;
        cz.part = b.part;
        cz.part_stride = b.part_stride;
        NUDIM_TRY(pl.adjoint(nplanes, sa, cz, st));
        int nxt = 1 - cur;
        launch_finish_sums(b.part, pl.crop_blocks(), nplanes, b.part_stride, b.dots + nxt, 4, 1,
                           st);
        // beta = |z'|^2/|z|^2; p = beta p + z'
        {
            ProfScope ps(pl.ctx, PK_CGVEC, st, 3.0 * sizeof(C) * (double)N * nplanes);
            dim3 gp(ceil_div(N, 256), nplanes);
            k_cg_pupdate<T><<<gp, 256, 0, st>>>(b.p, b.z, b.dots, cur, nxt, N);
            NUDIM_LAUNCH_CHECK();
        }
        cur = nxt;
    }
    return NUDIM_OK;
}

template int cgnr_run<double>(NfftDev<double> &, int, const double2 *, const double *,
                              double2 *, const double *, bool, int, CgnrBuffers<double> &,
                              cudaStream_t);
template int cgnr_run<float>(NfftDev<float> &, int, const float2 *, const float *, float2 *,
                             const float *, bool, int, CgnrBuffers<float> &, cudaStream_t);

// ================================================================ volume ops
// reconstruction.c:548-550: data[t] = img[(t + nz/2) % nz] (imaginary 0)
template <typename T>
__global__ void k_pack(const T *__restrict__ img, cplx_t<T> *__restrict__ data, int nz, size_t P2)
{
    int t = blockIdx.y;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P2) return;
    data[(size_t)t * P2 + i] = mkc<T>(img[(size_t)((t + nz / 2) % nz) * P2 + i], T(0));
}

// reconstruction.c:612-621: img[t] = Re(data[(t + nz/2) % nz]) / nz
template <typename T>
__global__ void k_unpack(const cplx_t<T> *__restrict__ data, T *__restrict__ img, int nz, size_t P2)
{
    int t = blockIdx.y;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P2) return;
    img[(size_t)t * P2 + i] = data[(size_t)((t + nz / 2) % nz) * P2 + i].x / (T)nz;
}

template <typename T> int launch_pack(const T *img, cplx_t<T> *data, int nz, size_t P2, cudaStream_t st)
{
    k_pack<T><<<dim3(ceil_div((long)P2, 256), nz), 256, 0, st>>>(img, data, nz, P2);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

template <typename T> int launch_unpack(const cplx_t<T> *data, T *img, int nz, size_t P2, cudaStream_t st)
{
    k_unpack<T><<<dim3(ceil_div((long)P2, 256), nz), 256, 0, st>>>(data, img, nz, P2);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

// reconstruction.c:672-700 / reconstruction-parallel.c:805-833.
// Inside the support u >= 0 is kept; u < 0 inside, and everything outside,
// becomes (HIO) img_last - 0.9 u or (ER) 0.  The result replaces img_last.
// The outer-iteration index lives on the device (set before each iteration)
// so that one captured graph serves every iteration.
__global__ void k_set_counter(int *it, int v) { *it = v; }

int launch_set_counter(int *it, int v, cudaStream_t st)
{
    k_set_counter<<<1, 1, 0, st>>>(it, v);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

template <typename T>
__global__ void k_constraint(const T *__restrict__ img, T *__restrict__ last, int np, int nx,
                             size_t P2, size_t V, const int *__restrict__ it, int nhio,
                             int height, int ylo, int yhi)
{
    size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= V) return;
    int hio = *it < nhio;
    size_t i = o % P2;
    int yi = (int)(i / np), xi = (int)(i % np);
    bool inside;
    if (height)
        inside = yi >= ylo && yi <= yhi;
    else
        inside = (yi >= (np - nx) / 2) && (yi < (np + nx) / 2) && (xi >= (np - nx) / 2) &&
                 (xi < (np + nx) / 2);
    T u = img[o];
    T out = u;
    if (!inside || u < T(0)) out = hio ? rn_sub(last[o], rn_mul((T)0.9, u)) : T(0);
    last[o] = out;
}

template <typename T>
int launch_constraint(T *img, const T *img_last, int nz, int np, int nx, const int *it,
                      int nhio, int height, int ylo, int yhi, cudaStream_t st)
{
    // img_last is overwritten with the constrained volume (it becomes the
    // next iteration's img and img_last).
    size_t P2 = (size_t)np * np, V = P2 * nz;
    k_constraint<T><<<ceil_div((long)V, 256), 256, 0, st>>>(img, (T *)img_last, np, nx, P2, V,
                                                            it, nhio, height, ylo, yhi);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

// R-factor of iteration nn: sqrt(sum diff1 / sum diff2) over planes
// (reconstruction.c:603-604), summed in plane order.
__global__ void k_finish_r(const double *__restrict__ d12, int nplanes, double *__restrict__ rh,
                           const int *__restrict__ it)
{
    int nn = *it;
    __shared__ double sh[32];
    double a = 0, c = 0;
    for (int p = threadIdx.x; p < nplanes; p += blockDim.x) {
        a += d12[2 * p];
        c += d12[2 * p + 1];
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) rh[nn] = sqrt(a / c);
}

template <typename T>
int launch_finish_r(const double *part, int nparts, int nplanes, int stride, double *rh,
                    const int *it, cudaStream_t st)
{
    // part holds per plane [nparts diff1 partials][nparts diff2 partials];
    // reduce them into d12 (stored after the partial area) then across planes.
    double *d12 = (double *)part + (size_t)nplanes * stride;
    launch_finish_sums(part, nparts, nplanes, stride, d12, 2, 2, st);
    k_finish_r<<<1, 256, 0, st>>>(d12, nplanes, rh, it);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

template <typename T> __global__ void k_real_to(const double *__restrict__ s, T *__restrict__ d, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = (T)s[i];
}

template <typename T> __global__ void k_to_double(const T *__restrict__ s, double *__restrict__ d, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = (double)s[i];
}

template <typename T> int launch_real_to(const double *src, T *dst, size_t n, cudaStream_t st)
{
    if (!n) return NUDIM_OK;
    k_real_to<T><<<ceil_div((long)n, 256), 256, 0, st>>>(src, dst, n);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

template <typename T> int launch_to_double(const T *src, double *dst, size_t n, cudaStream_t st)
{
    if (!n) return NUDIM_OK;
    k_to_double<T><<<ceil_div((long)n, 256), 256, 0, st>>>(src, dst, n);
    NUDIM_LAUNCH_CHECK();
    return NUDIM_OK;
}

#define NUDIM_INST(T)                                                                          \
    template int launch_pack<T>(const T *, cplx_t<T> *, int, size_t, cudaStream_t);           \
    template int launch_unpack<T>(const cplx_t<T> *, T *, int, size_t, cudaStream_t);         \
    template int launch_constraint<T>(T *, const T *, int, int, int, const int *, int, int,   \
                                      int, int, cudaStream_t);                                \
    template int launch_finish_r<T>(const double *, int, int, int, double *, const int *,     \
                                    cudaStream_t);                                            \
    template int launch_real_to<T>(const double *, T *, size_t, cudaStream_t);               \
    template int launch_to_double<T>(const T *, double *, size_t, cudaStream_t);
NUDIM_INST(double)
NUDIM_INST(float)

}  // namespace nudim
