// nfft.cu -- 2D NFFT forward (trafo) and adjoint on the GPU, batched over
// Z-planes.  Published method (Keiner, Kunis, Potts 2009): Kaiser-Bessel
// window, m = 6, oversampled grid n = 2 * next_pow2(N):
//   trafo   = D (deconvolve + pad) -> F (n0 x n1 FFT, cuFFT) -> B (interpolate)
//   adjoint = B^T (spread)        -> F^H                     -> D (crop + deconvolve)
// B is a gather from the oversampled grid (one thread per node); B^T is an
// atomic-free gather: every grid cell sums, in ascending node order, the
// nodes on its tile's list, so results are deterministic.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "engine.cuh"

namespace nudim {

// ================================================================ errors
static thread_local char g_err[512];

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char *last_error() { return g_err; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line)
{
    set_error("CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file,
              line);
    return e == cudaErrorMemoryAllocation ? NUDIM_ENOMEM : NUDIM_ECUDA;
}

int cufft_fail(cufftResult r, const char *what, const char *file, int line)
{
    set_error("cuFFT error %d in %s at %s:%d", (int)r, what, file, line);
    return r == CUFFT_ALLOC_FAILED ? NUDIM_ENOMEM : NUDIM_ECUDA;
}

unsigned long long g_launches = 0;

// ================================================================ profiler
static cudaEvent_t prof_event(nudim_ctx *c)
{
    if (!c->prof_pool.empty()) {
        cudaEvent_t e = c->prof_pool.back();
        c->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

ProfScope::ProfScope(nudim_ctx *c_, int k_, cudaStream_t st_, double bytes_)
    : c(c_), k(k_), st(st_), bytes(bytes_)
{
    if (c && c->prof_on) {
        a = prof_event(c);
        cudaEventRecord(a, st);
    }
}

ProfScope::~ProfScope()
{
    if (!a) return;
    cudaEvent_t b = prof_event(c);
    cudaEventRecord(b, st);
    c->prof_pending.push_back({k, a, b, bytes});
    if (c->prof_pending.size() > 4096) prof_collect(c);
}

int prof_collect(nudim_ctx *c)
{
    for (auto &r : c->prof_pending) {
        cudaEventSynchronize(r.b);
        float ms = 0;
        cudaEventElapsedTime(&ms, r.a, r.b);
        c->prof_ms[r.k] += ms;
        c->prof_n[r.k] += 1;
        c->prof_bytes[r.k] += r.bytes;
        c->prof_pool.push_back(r.a);
        c->prof_pool.push_back(r.b);
    }
    c->prof_pending.clear();
    return NUDIM_OK;
}

// ================================================================ context helpers
int ctx_workspace(nudim_ctx *ctx, size_t bytes, void **p)
{
    if (bytes > ctx->ws_bytes) {
        if (ctx->ws) {
            NUDIM_CUDA(cudaStreamSynchronize(ctx->stream));
            NUDIM_CUDA(cudaFree(ctx->ws));
            ctx->ws = nullptr;
            ctx->ws_bytes = 0;
        }
        NUDIM_CUDA(cudaMalloc(&ctx->ws, bytes));
        ctx->ws_bytes = bytes;
    }
    *p = ctx->ws;
    return NUDIM_OK;
}

int ctx_scratch(nudim_ctx *ctx, size_t bytes, double **p)
{
    if (bytes > ctx->scratch_bytes) {
        if (ctx->scratch) {
            NUDIM_CUDA(cudaStreamSynchronize(ctx->stream));
            NUDIM_CUDA(cudaFree(ctx->scratch));
            ctx->scratch = nullptr;
            ctx->scratch_bytes = 0;
        }
        NUDIM_CUDA(cudaMalloc(&ctx->scratch, bytes));
        ctx->scratch_bytes = bytes;
    }
    *p = ctx->scratch;
    return NUDIM_OK;
}

int ctx_fft2d(nudim_ctx *ctx, int n0, int n1, int batch, int prec, cufftHandle *h)
{
    auto key = std::make_tuple(n0, n1, batch, prec);
    auto it = ctx->fft2d.find(key);
    if (it != ctx->fft2d.end()) {
        *h = it->second;
        return NUDIM_OK;
    }
    cufftHandle p;
    int n[2] = {n0, n1};
    NUDIM_CUFFT(cufftPlanMany(&p, 2, n, nullptr, 1, n0 * n1, nullptr, 1, n0 * n1,
                              prec == NUDIM_FP64 ? CUFFT_Z2Z : CUFFT_C2C, batch));
    ctx->fft2d[key] = p;
    *h = p;
    return NUDIM_OK;
}

template <> int fft_exec<double>(cufftHandle h, double2 *io, int dir)
{
    NUDIM_CUFFT(cufftExecZ2Z(h, (cufftDoubleComplex *)io, (cufftDoubleComplex *)io, dir));
    return NUDIM_OK;
}
template <> int fft_exec<float>(cufftHandle h, float2 *io, int dir)
{
    NUDIM_CUFFT(cufftExecC2C(h, (cufftComplex *)io, (cufftComplex *)io, dir));
    return NUDIM_OK;
}

// ================================================================ reductions
__global__ void k_finish_sums(const double *__restrict__ part, int nparts, int stride_in,
                              double *__restrict__ out, int out_stride)
{
    __shared__ double sh[32];
    int b = blockIdx.x, k = blockIdx.y;
    const double *src = part + (size_t)b * stride_in + (size_t)k * nparts;
    double v = 0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += src[i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) out[(size_t)b * out_stride + k] = v;
}

void launch_finish_sums(const double *part, int nparts, int nplanes, int stride_in,
                        double *out, int out_stride, int nsums, cudaStream_t st)
{
    k_finish_sums<<<dim3(nplanes, nsums), 256, 0, st>>>(part, nparts, stride_in, out,
                                                         out_stride);
    ++g_launches;
}

// ================================================================ plan setup
// Stream-ordered upload of a host array (pageable sources are staged before
// cudaMemcpyAsync returns, so the host copy may be released right after).
int upload_async(void **dst, const void *src, size_t nb, cudaStream_t st)
{
    NUDIM_CUDA(cudaMallocAsync(dst, nb ? nb : 8, st));
    if (nb) NUDIM_CUDA(cudaMemcpyAsync(*dst, src, nb, cudaMemcpyHostToDevice, st));
    return NUDIM_OK;
}

template <typename T>
int NfftDev<T>::init(nudim_ctx *c, const NfftTables &t, cudaStream_t st, Workspace *w)
{
    ctx = c;
    wsp = w;
    ast = st;
    N0 = t.N0;
    N1 = t.N1;
    n0 = t.n0;
    n1 = t.n1;
    M = t.M;
    ty = t.ty;
    tx = t.tx;
    nty = t.nty;
    ntx = t.ntx;
    std::vector<int2> hu(M);
    for (int j = 0; j < M; j++) hu[j] = make_int2(t.u0[j], t.u1[j]);
    std::vector<T> hp(t.psi.begin(), t.psi.end());
    std::vector<T> hc0(t.c0.begin(), t.c0.end()), hc1(t.c1.begin(), t.c1.end());
    size_t nb_u = sizeof(int2) * (size_t)M, nb_p = sizeof(T) * hp.size();
    NUDIM_TRY(upload_async((void **)&u, hu.data(), nb_u, st));
    NUDIM_TRY(upload_async((void **)&psi, hp.data(), nb_p, st));
    NUDIM_TRY(upload_async((void **)&c0, hc0.data(), sizeof(T) * N0, st));
    NUDIM_TRY(upload_async((void **)&c1, hc1.data(), sizeof(T) * N1, st));
    bytes = nb_u + nb_p + sizeof(T) * (N0 + N1);
    // the fused path serves every geometry but extremely narrow grids, which
    // take the grid path below
    if (c->use_fused && c->autotune && !tune_bc && !tune_planes)
        NUDIM_TRY(autotune(t, st));
    if (c->use_fused && init_fused(t, st) == NUDIM_OK) return NUDIM_OK;
    fused = false;
    // grid path: tile lists of the spreading gather
    std::vector<int> toff, tnodes;
    build_tile_lists(t, &toff, &tnodes);
    if (tnodes.empty()) tnodes.assign(1, 0);
    NUDIM_TRY(upload_async((void **)&tile_off, toff.data(), sizeof(int) * toff.size(), st));
    NUDIM_TRY(upload_async((void **)&tile_nodes, tnodes.data(), sizeof(int) * tnodes.size(), st));
    bytes += sizeof(int) * (toff.size() + tnodes.size());
    return NUDIM_OK;
}

template <typename T> int NfftDev<T>::workspace(size_t nb, void **p)
{
    return wsp ? ws_get(wsp, nb, p) : ctx_workspace(ctx, nb, p);
}

int ws_get(Workspace *w, size_t bytes, void **out)
{
    if (bytes > w->bytes && w->frozen) {
        set_error("workspace of %zu bytes asked for %zu after a graph captured it", w->bytes,
                  bytes);
        return NUDIM_ESTATE;
    }
    if (bytes > w->bytes) {
        if (w->p) NUDIM_CUDA(cudaFreeAsync(w->p, w->st));
        w->p = nullptr;
        w->bytes = 0;
        NUDIM_CUDA(cudaMallocAsync(&w->p, bytes, w->st));
        w->bytes = bytes;
    }
    *out = w->p;
    return NUDIM_OK;
}

void ws_release(Workspace *w)
{
    if (w->p) cudaFreeAsync(w->p, w->st);
    w->p = nullptr;
    w->bytes = 0;
    w->frozen = false;
}

template <typename T> void NfftDev<T>::release()
{
    void *ptrs[] = {u, psi, c0, c1, tile_off, tile_nodes};
    for (void *q : ptrs)
        if (q) cudaFreeAsync(q, ast);
    u = nullptr;
    psi = nullptr;
    c0 = c1 = nullptr;
    tile_off = tile_nodes = nullptr;
    if (fused) release_fused();
}

template <typename T> int NfftDev<T>::chunk_for(int nplanes) const
{
    size_t per = sizeof(C) * (size_t)n0 * n1;
    size_t budget = ctx->grid_budget ? ctx->grid_budget : ((size_t)2 << 30);
    long c = (long)(budget / per);
    if (c < 1) c = 1;
    if (c > nplanes) c = nplanes;
    return (int)c;
}

// ================================================================ kernels
template <typename T, int MODE>
__global__ void __launch_bounds__(256)
k_pad(const void *__restrict__ src, size_t src_stride, int N0, int N1, int n0, int n1,
      const T *__restrict__ c0, const T *__restrict__ c1, int plane0,
      cplx_t<T> *__restrict__ grid, cplx_t<T> *__restrict__ f_init, size_t f_stride)
{
    using C = cplx_t<T>;
    int b = blockIdx.y;
    size_t cells = (size_t)n0 * n1;
    size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= cells) return;
    int l0 = (int)(cell / n1), l1 = (int)(cell % n1);
    int k0 = l0 < n0 / 2 ? l0 : l0 - n0;
    int k1 = l1 < n1 / 2 ? l1 : l1 - n1;
    C val = mkc<T>(0, 0);
    if (k0 >= -N0 / 2 && k0 < N0 / 2 && k1 >= -N1 / 2 && k1 < N1 / 2) {
        int a = k0 + N0 / 2, c = k1 + N1 / 2;
        size_t idx = (size_t)(plane0 + b) * src_stride + (size_t)a * N1 + c;
        C v;
        if (MODE == PM_COMPLEX) {
            v = ((const C *)src)[idx];
        } else {
            v = mkc<T>(((const T *)src)[idx], T(0));
            f_init[(size_t)(plane0 + b) * f_stride + (size_t)a * N1 + c] = v;
        }
        T s = c0[a] * c1[c];
        val = mkc<T>(v.x * s, v.y * s);
    }
    grid[(size_t)b * cells + cell] = val;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(256)
k_interp(const cplx_t<T> *__restrict__ grid, int n0, int n1, const int2 *__restrict__ u,
         const T *__restrict__ psi, int M, int plane0, InterpArgs<T> a)
{
    using C = cplx_t<T>;
    __shared__ double sh[32];
    int b = blockIdx.y, gb = plane0 + b;
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    const C *g = grid + (size_t)b * n0 * n1;
    T s0 = 0, s1 = 0;
    if (j < M) {
        int2 uu = u[j];
        const T *ps = psi + (size_t)j * 2 * kW;
        T p1[kW];
#pragma unroll
        for (int t = 0; t < kW; t++) p1[t] = ps[kW + t];
        T ar = 0, ai = 0;
        for (int t0 = 0; t0 < kW; t0++) {
            const C *row = g + (size_t)((uu.x + t0) & (n0 - 1)) * n1;
            T rr = 0, ri = 0;
#pragma unroll
            for (int t1 = 0; t1 < kW; t1++) {
                C v = __ldg(row + ((uu.y + t1) & (n1 - 1)));
                rr += p1[t1] * v.x;
                ri += p1[t1] * v.y;
            }
            T q = ps[t0];
            ar += q * rr;
            ai += q * ri;
        }
        C f = mkc<T>(ar, ai);
        size_t o = (size_t)gb * a.out_stride + j;
        if (MODE == IM_PLAIN) {
            a.out[o] = f;
        } else if (MODE == IM_RESID) {
            C yv = a.y[(size_t)gb * a.y_stride + j];
            a.out[o] = mkc<T>(yv.x - f.x, yv.y - f.y);
        } else if (MODE == IM_DOTV) {
            a.out[o] = f;
            T wv = a.w ? a.w[j] : T(1);
            s0 = wv * (f.x * f.x + f.y * f.y);
        } else {  // IM_CONSTRAINT: y = known ? s : f, R-factor partials
            if (a.known[j / a.line_len]) {
                C sv = a.s[(size_t)gb * a.s_stride + j];
                a.out[o] = sv;
                T dr = f.x - sv.x, di = f.y - sv.y, pr = f.x + sv.x, pi = f.y + sv.y;
                s0 = dr * dr + di * di;
                s1 = pr * pr + pi * pi;
            } else {
                a.out[o] = f;
            }
        }
    }
    if (MODE == IM_DOTV || MODE == IM_CONSTRAINT) {
        double v0 = block_sum_t<T>(s0, sh);
        if (threadIdx.x == 0) a.part[(size_t)gb * a.part_stride + blockIdx.x] = v0;
        if (MODE == IM_CONSTRAINT) {
            double v1 = block_sum_t<T>(s1, sh);
            if (threadIdx.x == 0)
                a.part[(size_t)gb * a.part_stride + gridDim.x + blockIdx.x] = v1;
        }
    }
}

constexpr int kSpreadChunk = 64;

template <typename T, bool WEIGHTED>
__global__ void __launch_bounds__(256)
k_spread(SpreadArgs<T> sa, const int2 *__restrict__ u, const T *__restrict__ psi,
         const int *__restrict__ tile_off, const int *__restrict__ tile_nodes, int n0, int n1,
         int ty, int tx, int ntx, int plane0, cplx_t<T> *__restrict__ grid)
{
    using C = cplx_t<T>;
    __shared__ int2 su[kSpreadChunk];
    __shared__ T sp[kSpreadChunk][2 * kW];
    __shared__ C sf[kSpreadChunk];
    int tile = blockIdx.x, b = blockIdx.y, gb = plane0 + b;
    int tr = tile / ntx, tc = tile % ntx;
    int r = tr * ty + threadIdx.x / tx, c = tc * tx + threadIdx.x % tx;
    int beg = tile_off[tile], end = tile_off[tile + 1];
    const C *f = sa.f + (size_t)gb * sa.f_stride;
    T ar = 0, ai = 0;
    Comp<T> kr, ki;  // compensated form for FP32
    kr.init();
    ki.init();
    for (int base = beg; base < end; base += kSpreadChunk) {
        int n = min(kSpreadChunk, end - base);
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            int j = tile_nodes[base + i];
            su[i] = u[j];
            C fv = f[j];
            if (WEIGHTED) {
                T wv = sa.w[j];
                fv = mkc<T>(wv * fv.x, wv * fv.y);
            }
            sf[i] = fv;
        }
        for (int i = threadIdx.x; i < n * 2 * kW; i += blockDim.x) {
            int q = i / (2 * kW), k = i - q * (2 * kW);
            sp[q][k] = psi[(size_t)tile_nodes[base + q] * 2 * kW + k];
        }
        __syncthreads();
        for (int i = 0; i < n; i++) {
            int d0 = (r - su[i].x) & (n0 - 1);
            if (d0 < kW) {
                int d1 = (c - su[i].y) & (n1 - 1);
                if (d1 < kW) {
                    T q0 = sp[i][d0], q1 = sp[i][kW + d1];
                    T vr = q1 * (q0 * sf[i].x), vi = q1 * (q0 * sf[i].y);
                    if (sizeof(T) == 4) {
                        kr.add(vr);
                        ki.add(vi);
                    } else {
                        ar += vr;
                        ai += vi;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (sizeof(T) == 4) {
        ar = kr.value();
        ai = ki.value();
    }
    grid[(size_t)b * n0 * n1 + (size_t)r * n1 + c] = mkc<T>(ar, ai);
}

template <typename T, int MODE>
__global__ void __launch_bounds__(256)
k_crop(const cplx_t<T> *__restrict__ grid, int n0, int n1, int N0, int N1,
       const T *__restrict__ c0, const T *__restrict__ c1, int plane0, CropArgs<T> a)
{
    using C = cplx_t<T>;
    __shared__ double sh[32];
    int b = blockIdx.y, gb = plane0 + b;
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t NN = (size_t)N0 * N1;
    T s = 0;
    if (k < NN) {
        int ai = (int)(k / N1), ci = (int)(k % N1);
        int l0 = (ai - N0 / 2) & (n0 - 1), l1 = (ci - N1 / 2) & (n1 - 1);
        C g = grid[(size_t)b * n0 * n1 + (size_t)l0 * n1 + l1];
        T sc = c0[ai] * c1[ci];
        C z = mkc<T>(g.x * sc, g.y * sc);
        a.out[(size_t)gb * a.out_stride + k] = z;
        if (MODE == CM_INIT) a.p_out[(size_t)gb * a.out_stride + k] = z;
        s = z.x * z.x + z.y * z.y;
    }
    if (MODE != CM_PLAIN) {
        double d = block_sum_t<T>(s, sh);
        if (threadIdx.x == 0) a.part[(size_t)gb * a.part_stride + blockIdx.x] = d;
    }
}

// ================================================================ drivers
// Algorithmic bytes per launch (profiler): c = complex size, T = real size.
//   pad    nb*c*(N0*N1 + n0*n1)             read coefficients, write grid
//   fft2d  nb*c*2*n0*n1                      one read + one write of the grid
//   interp M*(8+2kW*T) + nb*c*(n0*n1 + M)    node tables once, grid, output
//   spread M*(8+2kW*T) + nb*c*(M + n0*n1)    node tables once, input, grid
//   crop   nb*c*2*N0*N1                      read window of grid, write result
template <typename T>
int NfftDev<T>::trafo(int nplanes, const PadArgs<T> &pa, const InterpArgs<T> &ia,
                      cudaStream_t st)
{
    if (nplanes <= 0) return NUDIM_OK;
    if (fused) return trafo_fused(nplanes, pa, ia, st);
    int chunk = chunk_for(nplanes);
    void *wsv;
    NUDIM_TRY(workspace(sizeof(C) * (size_t)n0 * n1 * chunk, &wsv));
    C *grid = (C *)wsv;
    size_t cells = (size_t)n0 * n1;
    const double c = sizeof(C), tab = (double)M * (8 + 2 * kW * sizeof(T));
    for (int p0 = 0; p0 < nplanes; p0 += chunk) {
        int nb = std::min(chunk, nplanes - p0);
        {
            ProfScope ps(ctx, PK_PAD, st, nb * c * ((double)N0 * N1 + (double)cells));
            dim3 gpad(ceil_div((long)cells, 256), nb);
            if (pa.mode == PM_COMPLEX)
                k_pad<T, PM_COMPLEX><<<gpad, 256, 0, st>>>(pa.src, pa.src_stride, N0, N1, n0, n1,
                                                           c0, c1, p0, grid, nullptr, 0);
            else
                k_pad<T, PM_REAL_INIT><<<gpad, 256, 0, st>>>(pa.src, pa.src_stride, N0, N1, n0,
                                                             n1, c0, c1, p0, grid, pa.f_init,
                                                             pa.f_stride);
            NUDIM_LAUNCH_CHECK();
        }
        {
            ProfScope ps(ctx, PK_FFT2D, st, nb * c * 2.0 * (double)cells);
            cufftHandle h;
            NUDIM_TRY(ctx_fft2d(ctx, n0, n1, nb, prec_of<T>(), &h));
            NUDIM_CUFFT(cufftSetStream(h, st));
            NUDIM_TRY(fft_exec<T>(h, grid, CUFFT_FORWARD));
        }
        {
            ProfScope ps(ctx, PK_INTERP, st, tab + nb * c * ((double)cells + M));
            dim3 gi(interp_blocks(), nb);
            switch (ia.mode) {
            case IM_PLAIN: k_interp<T, IM_PLAIN><<<gi, 256, 0, st>>>(grid, n0, n1, u, psi, M, p0, ia); break;
            case IM_RESID: k_interp<T, IM_RESID><<<gi, 256, 0, st>>>(grid, n0, n1, u, psi, M, p0, ia); break;
            case IM_DOTV: k_interp<T, IM_DOTV><<<gi, 256, 0, st>>>(grid, n0, n1, u, psi, M, p0, ia); break;
            default: k_interp<T, IM_CONSTRAINT><<<gi, 256, 0, st>>>(grid, n0, n1, u, psi, M, p0, ia); break;
            }
            NUDIM_LAUNCH_CHECK();
        }
    }
    return NUDIM_OK;
}

template <typename T>
int NfftDev<T>::adjoint(int nplanes, const SpreadArgs<T> &sa, const CropArgs<T> &ca,
                        cudaStream_t st)
{
    if (nplanes <= 0) return NUDIM_OK;
    if (fused) return adjoint_fused(nplanes, sa, ca, st);
    int chunk = chunk_for(nplanes);
    void *wsv;
    NUDIM_TRY(workspace(sizeof(C) * (size_t)n0 * n1 * chunk, &wsv));
    C *grid = (C *)wsv;
    const double c = sizeof(C), cells = (double)n0 * n1,
                 tab = (double)M * (8 + 2 * kW * sizeof(T));
    for (int p0 = 0; p0 < nplanes; p0 += chunk) {
        int nb = std::min(chunk, nplanes - p0);
        {
            ProfScope ps(ctx, PK_SPREAD, st, tab + nb * c * ((double)M + cells));
            dim3 gs(nty * ntx, nb);
            if (sa.w)
                k_spread<T, true><<<gs, ty * tx, 0, st>>>(sa, u, psi, tile_off, tile_nodes, n0,
                                                          n1, ty, tx, ntx, p0, grid);
            else
                k_spread<T, false><<<gs, ty * tx, 0, st>>>(sa, u, psi, tile_off, tile_nodes, n0,
                                                           n1, ty, tx, ntx, p0, grid);
            NUDIM_LAUNCH_CHECK();
        }
        {
            ProfScope ps(ctx, PK_FFT2D, st, nb * c * 2.0 * cells);
            cufftHandle h;
            NUDIM_TRY(ctx_fft2d(ctx, n0, n1, nb, prec_of<T>(), &h));
            NUDIM_CUFFT(cufftSetStream(h, st));
            NUDIM_TRY(fft_exec<T>(h, grid, CUFFT_INVERSE));
        }
        {
            ProfScope ps(ctx, PK_CROP, st, nb * c * 2.0 * N0 * N1);
            dim3 gc(crop_blocks(), nb);
            switch (ca.mode) {
            case CM_PLAIN: k_crop<T, CM_PLAIN><<<gc, 256, 0, st>>>(grid, n0, n1, N0, N1, c0, c1, p0, ca); break;
            case CM_DOT: k_crop<T, CM_DOT><<<gc, 256, 0, st>>>(grid, n0, n1, N0, N1, c0, c1, p0, ca); break;
            default: k_crop<T, CM_INIT><<<gc, 256, 0, st>>>(grid, n0, n1, N0, N1, c0, c1, p0, ca); break;
            }
            NUDIM_LAUNCH_CHECK();
        }
    }
    return NUDIM_OK;
}

template struct NfftDev<double>;
template struct NfftDev<float>;

}  // namespace nudim
