// denoise.cu -- TV-discrete (and its height-window variant) and the in-place
// 2D anisotropic diffusion of denoise.c, on [z][y][x] volumes.
//
// Arithmetic uses round-to-nearest intrinsics (no contraction) so that the
// FP64 form reproduces the reference's per-voxel C arithmetic exactly; only
// the two global sums of TV are summed in a different (tree) order.  The
// FP32 form uses fused multiply-adds, rsqrt and fast division where noted.
#include "engine.cuh"

#include <cstdlib>
#include <cstring>
#include <type_traits>

namespace nudim {

// ================================================================ TV
// denoise.c:67-151 / 153-249 called as total_variation_discrete(img, lam,
// niter, nz, np, np): the reference's i runs over Z, j over Y, k over X.
//
// One TV iteration is two launches:
//   k_tv_grad   the gradient g of every voxel and the two global sums
//               (sum g^2, sum of squares of the negative voxels).  A block
//               owns a 32 x 16 (x, y) tile and a run of Z-planes; it marches
//               along Z with three planes of the tile plus a one-cell halo in
//               shared memory, so every voxel is read from memory about once.
//               The halo cells hold the clamped neighbours (index -1 -> 0,
//               n -> n-1), which are exactly the reference's boundary rules.
//               The block that finishes last sums the per-block partials in
//               block order (deterministic) into scal[0..1];
//   k_tv_update u -= (lam sqrt(scal[1])) (g / sqrt(scal[0])).
constexpr int kTvTX = 32, kTvTY = 16, kTvSX = kTvTX + 2, kTvSY = kTvTY + 2;
constexpr int kTvRows = kTvTY / 8;  // rows per thread (256 threads = 8 warps of 32 x)

// Gradient of voxel (i, j, k) (denoise.c:84-122) from three tile planes:
// p = plane clamp(i-1), q = plane i, r = plane clamp(i+1), the voxel at
// tile cell (y, x); the reference's IEEE operations in its order (the FP64
// form; the FP32 form runs tv_point2).
template <typename T>
__device__ __forceinline__ T tv_point(const T (*p)[kTvSX], const T (*q)[kTvSX],
                                      const T (*r)[kTvSX], int y, int x, T &c)
{
    const T eps = (T)1e-8;
    c = q[y][x];
    T t1 = rn_sub(c, p[y][x]);
    T t2 = rn_sub(c, q[y - 1][x]);
    T t3 = rn_sub(c, q[y][x - 1]);
    T a4 = r[y][x];
    T t4 = rn_sub(a4, c);
    T t5 = rn_sub(a4, r[y - 1][x]);
    T t6 = rn_sub(a4, r[y][x - 1]);
    T a7 = q[y + 1][x];
    T t7 = rn_sub(a7, p[y + 1][x]);
    T t8 = rn_sub(a7, c);
    T t9 = rn_sub(a7, q[y + 1][x - 1]);
    T a10 = q[y][x + 1];
    T t10 = rn_sub(a10, p[y][x + 1]);
    T t11 = rn_sub(a10, q[y - 1][x + 1]);
    T t12 = rn_sub(a10, c);
    auto nrm = [&](T x, T y, T z) {
        return rn_sqrt(rn_add(rn_add(rn_add(eps, rn_mul(x, x)), rn_mul(y, y)), rn_mul(z, z)));
    };
    T g1 = rn_div(rn_add(rn_add(t1, t2), t3), nrm(t1, t2, t3));
    T g2 = rn_div(t4, nrm(t4, t5, t6));
    T g3 = rn_div(t8, nrm(t7, t8, t9));
    T g4 = rn_div(t12, nrm(t10, t11, t12));
    return rn_sub(rn_sub(rn_sub(g1, g2), g3), g4);
}

// FP32 form, two voxels at once: tile cells (y, x) and (y + 8, x), each
// operation paired (one paired add / fused multiply-add / multiply for both
// voxels); t / sqrt(eps + x^2 + y^2 + z^2) as t * rsqrt(...) with fused
// multiply-adds (a few ulp per term, against one for IEEE sqrt and division;
// the TV loop's own amplification of rounding dominates).  c returns both
// centre values.
__device__ __forceinline__ float2 tv_point2(const float (*p)[kTvSX], const float (*q)[kTvSX],
                                            const float (*r)[kTvSX], int y, int x, float2 &c)
{
    auto ld = [&](const float (*a)[kTvSX], int yy, int xx) {
        return make_float2(a[yy][xx], a[yy + 8][xx]);
    };
    auto sub = [](float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); };
    c = ld(q, y, x);
    const float2 t1 = sub(c, ld(p, y, x)), t2 = sub(c, ld(q, y - 1, x)),
                 t3 = sub(c, ld(q, y, x - 1));
    const float2 a4 = ld(r, y, x);
    const float2 t4 = sub(a4, c), t5 = sub(a4, ld(r, y - 1, x)), t6 = sub(a4, ld(r, y, x - 1));
    const float2 a7 = ld(q, y + 1, x);
    const float2 t7 = sub(a7, ld(p, y + 1, x)), t8 = sub(a7, c),
                 t9 = sub(a7, ld(q, y + 1, x - 1));
    const float2 a10 = ld(q, y, x + 1);
    const float2 t10 = sub(a10, ld(p, y, x + 1)), t11 = sub(a10, ld(q, y - 1, x + 1)),
                 t12 = sub(a10, c);
    const float2 e2 = make_float2(1e-8f, 1e-8f);
    auto inv = [&](float2 a, float2 b, float2 d) {
        float2 s = __ffma2_rn(d, d, __ffma2_rn(b, b, __ffma2_rn(a, a, e2)));
        return make_float2(rsqrtf(s.x), rsqrtf(s.y));
    };
    const float2 h1 = __fmul2_rn(__fadd2_rn(__fadd2_rn(t1, t2), t3), inv(t1, t2, t3));
    const float2 h2 = __fmul2_rn(t4, inv(t4, t5, t6));
    const float2 h3 = __fmul2_rn(t8, inv(t7, t8, t9));
    const float2 h4 = __fmul2_rn(t12, inv(t10, t11, t12));
    return sub(sub(sub(h1, h2), h3), h4);
}

// A thread's running sum of its voxels' terms: plain in the FP64 form,
// Neumaier-compensated in the FP32 form (a thread sums one term per plane of
// its Z-run).
template <typename T> struct TvAcc {
    T s = 0, e = 0;
    __device__ __forceinline__ void add(T x)
    {
        if (sizeof(T) == 8) {
            s = rn_add(s, x);
            return;
        }
        T t = rn_add(s, x);
        e = rn_add(e, fabs(s) >= fabs(x) ? rn_add(rn_sub(s, t), x) : rn_add(rn_sub(x, t), s));
        s = t;
    }
    __device__ __forceinline__ T value() const { return rn_add(s, e); }
};

// The two sums: FP64 products and sums in the FP64 form; FP32 products and
// compensated per-thread sums, FP32 warp sums and FP64 across warps and
// blocks in the FP32 form.  Grid (x tiles, y tiles, Z-runs of zc planes);
// 256 threads, thread (ty, tx) owns the columns (j0 + ty + 8 r, k0 + tx),
// r < kTvRows.  done: a zeroed counter (the last block resets it).
//
// FUSED: the previous iteration's update is applied as the tile is read
// (u' = u - (lam sqrt(scal_in[1])) (g_in / sqrt(scal_in[0])) on every tile
// and halo cell, with k_tv_update's operations), the owned cells' u' are
// written to u_out and the gradient of u' to g: one pass reads u and g_in and
// writes u' and g (4 values per voxel instead of the 5 of a gradient and an
// update).  u_out and g must not alias u and g_in (other blocks still read
// their halos).
template <typename T, bool FUSED>
__global__ void __launch_bounds__(256)
k_tv_grad(const T *__restrict__ u, T *__restrict__ g, double *__restrict__ part,
          unsigned *__restrict__ done, double *__restrict__ scal, int nz, int ny, int nx,
          int zc, int height, int ylo, int yhi, const T *__restrict__ g_in,
          const double *__restrict__ scal_in, double lam, T *__restrict__ u_out)
{
    constexpr int kCells = kTvSY * kTvSX, kSlots = (kCells + 255) / 256;
    __shared__ T pl[3][kTvSY][kTvSX];
    __shared__ double sh[32];
    __shared__ int s_last;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int k0 = blockIdx.x * kTvTX, j0 = blockIdx.y * kTvTY;
    const int z0 = blockIdx.z * zc, z1 = min(nz, z0 + zc);
    const int k = k0 + tx;
    bool own[kTvRows], inb[kTvRows];
#pragma unroll
    for (int r = 0; r < kTvRows; r++) {
        const int j = j0 + ty + 8 * r;
        inb[r] = k < nx && j < ny;
        own[r] = inb[r] && (!height || (j >= ylo && j <= yhi));
    }
    const size_t P = (size_t)ny * nx;
    // this thread's halo-tile cells, their clamped in-plane offsets and (FUSED)
    // whether the update applies to their row
    int cell[kSlots];
    size_t off[kSlots];
    bool upd[kSlots];
#pragma unroll
    for (int s = 0; s < kSlots; s++) {
        int c = threadIdx.x + 256 * s;
        cell[s] = c < kCells ? c : -1;
        int yy = c / kTvSX, xx = c - yy * kTvSX;
        int gj = min(max(j0 + yy - 1, 0), ny - 1), gk = min(max(k0 + xx - 1, 0), nx - 1);
        off[s] = (size_t)gj * nx + gk;
        upd[s] = !height || (gj >= ylo && gj <= yhi);
    }
    T tn = T(1), la = T(0);
    if (FUSED) {  // the same FP64 expressions as k_tv_update
        tn = (T)sqrt(scal_in[0]);
        la = (T)(lam * sqrt(scal_in[1]));
    }
    T pre[kSlots], preg[kSlots];
    auto fetch = [&](int plane) {
#pragma unroll
        for (int s = 0; s < kSlots; s++)
            if (cell[s] >= 0) {
                pre[s] = u[(size_t)plane * P + off[s]];
                if (FUSED) preg[s] = g_in[(size_t)plane * P + off[s]];
            }
    };
    auto store = [&](int b) {
#pragma unroll
        for (int s = 0; s < kSlots; s++)
            if (cell[s] >= 0) {
                T v = pre[s];
                if (FUSED && upd[s]) v = rn_sub(v, rn_mul(la, rn_div(preg[s], tn)));
                (&pl[b][0][0])[cell[s]] = v;
            }
    };
    int bp = 0, bc = 1, bn = 2;
    fetch(max(z0 - 1, 0));
    store(bp);
    fetch(z0);
    store(bc);
    fetch(min(z0 + 1, nz - 1));
    store(bn);
    __syncthreads();
    TvAcc<T> ag, an;
    for (int i = z0; i < z1; i++) {
        if (i + 1 < z1) fetch(min(i + 2, nz - 1));  // in flight during the compute
        if constexpr (sizeof(T) == 4 && kTvRows == 2) {
            float2 c2;
            const float2 g2 = tv_point2(pl[bp], pl[bc], pl[bn], ty + 1, tx + 1, c2);
            const float gv[2] = {g2.x, g2.y}, cv[2] = {c2.x, c2.y};
#pragma unroll
            for (int r = 0; r < 2; r++) {
                if (FUSED && inb[r]) u_out[(size_t)i * P + (size_t)(j0 + ty + 8 * r) * nx + k] = cv[r];
                if (own[r]) {
                    g[(size_t)i * P + (size_t)(j0 + ty + 8 * r) * nx + k] = gv[r];
                    ag.add(rn_mul(gv[r], gv[r]));
                    if (cv[r] < 0.f) an.add(rn_mul(cv[r], cv[r]));
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < kTvRows; r++) {
                if (FUSED && inb[r])
                    u_out[(size_t)i * P + (size_t)(j0 + ty + 8 * r) * nx + k] =
                        pl[bc][ty + 8 * r + 1][tx + 1];
                if (own[r]) {
                    T c;
                    T gv = tv_point<T>(pl[bp], pl[bc], pl[bn], ty + 8 * r + 1, tx + 1, c);
                    g[(size_t)i * P + (size_t)(j0 + ty + 8 * r) * nx + k] = gv;
                    ag.add(rn_mul(gv, gv));
                    if (c < T(0)) an.add(rn_mul(c, c));
                }
            }
        }
        __syncthreads();
        if (i + 1 < z1) {
            int t = bp;
            bp = bc;
            bc = bn;
            bn = t;
            store(bn);
            __syncthreads();
        }
    }
    const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    double bg = block_sum_t<T>(ag.value(), sh);
    double bn2 = block_sum_t<T>(an.value(), sh);
    if (threadIdx.x == 0) {
        part[bid] = bg;
        part[nblk + bid] = bn2;
        __threadfence();
        s_last = atomicAdd(done, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!s_last) return;
    // the last block: every block's partials are visible (fence before the
    // count); sum them in block order, the same order whichever block is last
    __threadfence();
    double a = 0, b = 0;
    for (int t = threadIdx.x; t < (int)nblk; t += blockDim.x) {
        a += __ldcg(part + t);
        b += __ldcg(part + nblk + t);
    }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) {
        scal[0] = a;
        scal[1] = b;
        *done = 0;
    }
}

template <typename T, int N> struct alignas(sizeof(T) * N) TvVec {
    T v[N];
};

// u_out = u - (lam * sqrt(dA)) * (g / sqrt(sum g^2))   (denoise.c:125-142),
// VEC voxels per access; u_out may be u.  The two scalars are formed once per
// block (the same FP64 expressions in every block, so every voxel sees the
// same values).
template <typename T, typename I, int VEC>
__global__ void __launch_bounds__(256)
k_tv_update(const T *u, T *u_out, const T *__restrict__ g, const double *__restrict__ scal,
            double lam, int nz, int ny, int nx, int height, int ylo, int yhi)
{
    __shared__ T s_tn, s_la;
    if (threadIdx.x == 0) {
        s_tn = (T)sqrt(scal[0]);
        s_la = (T)(lam * sqrt(scal[1]));
    }
    __syncthreads();
    const T tn = s_tn, la = s_la;
    const I nv = (I)nz * ny * nx / VEC, stride = (I)gridDim.x * blockDim.x;
    for (I t = (I)blockIdx.x * blockDim.x + threadIdx.x; t < nv; t += stride) {
        TvVec<T, VEC> x = reinterpret_cast<const TvVec<T, VEC> *>(u)[t];
        const TvVec<T, VEC> y = reinterpret_cast<const TvVec<T, VEC> *>(g)[t];
#pragma unroll
        for (int e = 0; e < VEC; e++) {
            if (height) {
                int j = (int)(((t * VEC + e) / (I)nx) % (I)ny);
                if (j < ylo || j > yhi) continue;
            }
            x.v[e] = rn_sub(x.v[e], rn_mul(la, rn_div(y.v[e], tn)));
        }
        reinterpret_cast<TvVec<T, VEC> *>(u_out)[t] = x;
    }
}

// Per-block partial sums of k_tv_grad (two per block; at most one block per
// tile and plane) and the completion counter.
int tv_part_count(int nz, int ny, int nx)
{
    return 2 * ceil_div(nx, kTvTX) * ceil_div(ny, kTvTY) * nz + 2;
}

template <typename T> static int tv_grad_blocks_per_sm()
{
    static const int occ = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_tv_grad<T, true>, 256, 0) !=
                cudaSuccess ||
            b < 1)
            b = 1;
        return b;
    }();
    return occ;
}

// Fused passes (FP32 default) or a gradient and a separate update per
// iteration (FP64 default: the FP64 gradient is bound by the FP64 pipe, and
// the folded update made it slower than the two launches); NUDIM_TV=
// fused|unfused selects one.  The same values bit for bit; read at every call.
template <typename T> static bool tv_unfused()
{
    const char *e = getenv("NUDIM_TV");
    if (e && !strcmp(e, "unfused")) return true;
    if (e && !strcmp(e, "fused")) return false;
    return sizeof(T) == 8;
}

template <typename T, typename I>
static int tv_launch(T *u, T *grad, double *part, int part_cap, double *scal, size_t V, int nz,
                     int ny, int nx, float lam, int niter, int height, int ylo, int yhi,
                     T *u2, T *g2, cudaStream_t st)
{
    int dev = 0, sms = 0;
    NUDIM_CUDA(cudaGetDevice(&dev));
    NUDIM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // Z-runs: about two resident waves of blocks, runs of at least 4 planes
    // (each run re-reads two planes beyond its ends)
    const long tiles = (long)ceil_div(nx, kTvTX) * ceil_div(ny, kTvTY);
    const long want = 2L * sms * tv_grad_blocks_per_sm<T>();
    const int runs = (int)std::max(1L, std::min((long)nz / 4, (long)ceil_div(want, tiles)));
    const int zc = ceil_div(nz, runs);
    const dim3 gg(ceil_div(nx, kTvTX), ceil_div(ny, kTvTY), ceil_div(nz, zc));
    const long nb = (long)gg.x * gg.y * gg.z;
    if (part_cap < 2 * nb + 1) {
        set_error("tv_run: partial buffer too small");
        return NUDIM_EINVAL;
    }
    unsigned *done = reinterpret_cast<unsigned *>(part + 2 * nb);
    NUDIM_CUDA(cudaMemsetAsync(done, 0, sizeof(unsigned), st));
    constexpr int W = 16 / sizeof(T);
    const long nu1 = std::min((long)ceil_div((long)V, 256), (long)sms * 8);
    const long nuw = std::min((long)ceil_div((long)(V / W), 256), (long)sms * 8);
    auto wide = [&](const T *a, const T *b, const T *c) {
        return V % W == 0 && (reinterpret_cast<uintptr_t>(a) % 16) == 0 &&
               (reinterpret_cast<uintptr_t>(b) % 16) == 0 &&
               (reinterpret_cast<uintptr_t>(c) % 16) == 0;
    };
    // u_out = u - step(g, scal): the widest access that divides the volume and
    // the pointers' alignment
    auto update = [&](const T *uin, T *uout, const T *gv, const double *sc) -> int {
        if (wide(uin, uout, gv))
            k_tv_update<T, I, W><<<(int)nuw, 256, 0, st>>>(uin, uout, gv, sc, (double)lam, nz, ny,
                                                            nx, height, ylo, yhi);
        else
            k_tv_update<T, I, 1><<<(int)nu1, 256, 0, st>>>(uin, uout, gv, sc, (double)lam, nz, ny,
                                                            nx, height, ylo, yhi);
        NUDIM_LAUNCH_CHECK();
        return NUDIM_OK;
    };
    if (niter <= 0) return NUDIM_OK;
    if (!u2 || !g2 || niter < 2 || tv_unfused<T>()) {
        for (int it = 0; it < niter; it++) {
            k_tv_grad<T, false><<<gg, 256, 0, st>>>(u, grad, part, done, scal, nz, ny, nx, zc,
                                                    height, ylo, yhi, nullptr, nullptr, 0.0,
                                                    nullptr);
            NUDIM_LAUNCH_CHECK();
            NUDIM_TRY(update(u, u, grad, scal));
        }
        return NUDIM_OK;
    }
    // fused: the gradient of u, then niter - 1 passes that update with the
    // previous gradient and take the next one (volumes and gradients alternate
    // between (u, grad) and (u2, g2), the sums between scal[0..1] and
    // scal[2..3]), then the last update into u
    k_tv_grad<T, false><<<gg, 256, 0, st>>>(u, grad, part, done, scal, nz, ny, nx, zc, height, ylo,
                                            yhi, nullptr, nullptr, 0.0, nullptr);
    NUDIM_LAUNCH_CHECK();
    T *cu = u, *cg = grad;
    double *cs = scal;
    for (int it = 1; it < niter; it++) {
        T *nu = cu == u ? u2 : u, *ng = cg == grad ? g2 : grad;
        double *ns = cs == scal ? scal + 2 : scal;
        k_tv_grad<T, true><<<gg, 256, 0, st>>>(cu, ng, part, done, ns, nz, ny, nx, zc, height, ylo,
                                               yhi, cg, cs, (double)lam, nu);
        NUDIM_LAUNCH_CHECK();
        cu = nu;
        cg = ng;
        cs = ns;
    }
    return update(cu, u, cg, cs);
}

template <typename T>
int tv_run(T *u, T *grad, double *part, int part_cap, double *scal, int nz, int ny, int nx,
           float lam, int niter, int height, int ylo, int yhi, cudaStream_t st, T *u2, T *g2)
{
    size_t V = (size_t)nz * ny * nx;
    if (V == 0 || niter <= 0) return NUDIM_OK;
    // 32-bit voxel indices while index + grid stride stays below 2^32
    if (V < ((size_t)1 << 31))
        return tv_launch<T, unsigned>(u, grad, part, part_cap, scal, V, nz, ny, nx, lam, niter,
                                      height, ylo, yhi, u2, g2, st);
    return tv_launch<T, size_t>(u, grad, part, part_cap, scal, V, nz, ny, nx, lam, niter, height,
                                ylo, yhi, u2, g2, st);
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
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float diff_coef(float g, float Ksq)
{
    return Ksq * rcp_approx(fmaf(g, g, Ksq));
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
// per step.  The cells of a step are dealt out as 128-cell segments of the
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
    // prefix count of its 128-cell tasks, d, y0(d), len(d), and the ring offsets
    // of diagonals d, d - 1, d + 1
    constexpr int TC = 128;
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
            // slots a diagonal of this plane can use (uniform: a real branch)
            const int npf = (L + blockDim.x - 1) / blockDim.x;
            T pf[kDiffPf];
#pragma unroll
            for (int k = 0; k < kDiffPf; k++) {
                if (k >= npf) break;
                int i = threadIdx.x + k * blockDim.x;
                pf[k] = i < nn ? U[cell(dn, i)] : T(0);
            }
            // the next step's task table (warp 0), then this step's tasks:
            // 128-cell segments of the active diagonals, dealt out to the warps
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
                    if (k >= npf) break;
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

// The same ring of diagonals with the work dealt out by rows instead of task
// tables.  A slot holds a diagonal at its rows' positions (cell (y, d - y) of
// diagonal d at position y of slot d mod R, slots ny values long), so a cell's
// N and W sit at y - 1 and y of slot d - 1 and its S and E at y + 1 and y of
// slot d + 1.  At step t sweep g updates row y's cell on diagonal t - 2g.  A
// warp owns 32 consecutive rows and one of TPR sweep classes (g = class mod
// TPR): at a given sweep its lanes touch consecutive positions of one slot
// (no bank conflicts), and no per-step table or search is needed.  (Tried
// and slower, measured: classes re-dealt per step to the rows a step has,
// and two cells per iteration with paired FP32 arithmetic.)  Prefetch of
// diagonal t + 2, write-back of the group's final diagonal and one barrier
// per step as in k_diffusion_ring.  Requires min(ny, nx) <= kDiffPf *
// blockDim.x, blockDim.x a multiple of 32 TPR and, FP32, blockDim.x <= 768
// (two CTAs per SM).
template <typename T> struct DiffNb {
    T c, n, w, s, e;
};

template <typename T, int TPR>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 768 : 1024, sizeof(T) == 4 ? 2 : 1)
k_diffusion_rows(T *u, int ny, int nx, int nxb, double lambda_d, double ksq_d, int niter,
                 int G, int R)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T *ring = (T *)smraw;
    T *U = u + (size_t)blockIdx.x * ny * nx;
    const T lambda = (T)lambda_d, Ksq = (T)ksq_d;
    const int D = ny + nx - 1, L = min(ny, nx);
    auto y0 = [&](int d) { return max(0, d - (nx - 1)); };
    auto len = [&](int d) { return min(d, ny - 1) - y0(d) + 1; };
    // position i (row y0(d) + i) of diagonal d in the ring, and in the plane
    auto slot = [&](int d) { return ring + (size_t)(d % R) * ny + y0(d); };
    auto cell = [&](int d, int i) -> size_t {
        int a = y0(d);
        return (size_t)(a + i) * nx + (d - a - i);
    };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cls = warp % TPR;
    const int yfirst = (warp / TPR) * 32 + lane, ystride = blockDim.x / TPR;
    const int dstep = (2 * TPR) % R;  // ring slots between sweeps g and g + TPR
    // one cell's values: (y, x) of the diagonal in slot sd.  The reference's
    // clamps (denoise.c:343-351): a clamped neighbour is the cell itself,
    // x + 1 == nx reads 0.0; the reads a clamp replaces stay inside their
    // slots and are discarded.
    auto load = [&](int sd, int y, int x, bool hasN, bool hasS, int yN, int yS) {
        const int sm = sd == 0 ? R - 1 : sd - 1, sp = sd == R - 1 ? 0 : sd + 1;
        const T *rc = ring + sd * ny, *rm = ring + sm * ny, *rp = ring + sp * ny;
        DiffNb<T> v;
        v.c = rc[y];
        const T vN = rm[yN], vW = rm[y], vS = rp[yS], vE = rp[y];
        v.n = hasN ? vN : v.c;
        v.w = x > 0 ? vW : v.c;
        v.s = hasS ? vS : v.c;
        v.e = x == nxb - 1 ? v.c : (x + 1 < nx ? vE : T(0));
        return v;
    };
    for (int s0 = 0; s0 < niter; s0 += G) {
        const int gc = min(G, niter - s0);
        const int nsteps = D + 2 * (gc - 1);
        for (int d = 0; d < 2 && d < D; d++) {
            T *sd = slot(d);
            for (int i = threadIdx.x; i < len(d); i += blockDim.x) sd[i] = U[cell(d, i)];
        }
        __syncthreads();
        for (int t = 0; t < nsteps; t++) {
            // fetch diagonal t + 2 (stored after this step's cells)
            const int dn = t + 2;
            const int nn = dn < D ? len(dn) : 0;
            const int npf = (L + blockDim.x - 1) / blockDim.x;
            T pf[kDiffPf];
#pragma unroll
            for (int k = 0; k < kDiffPf; k++) {
                if (k >= npf) break;
                const int i = threadIdx.x + k * blockDim.x;
                pf[k] = i < nn ? U[cell(dn, i)] : T(0);
            }
            if (cls < gc)
                for (int y = yfirst; y <= t && y < ny; y += ystride) {
                    // this class's sweeps with a cell in row y: x = t - y - 2g
                    // in [0, nx - 1] and g < gc
                    const int ghi = min(gc - 1, (t - y) >> 1);
                    int glo = t - y - nx + 2;
                    glo = glo > 0 ? glo >> 1 : 0;
                    int g = glo + ((cls - glo) % TPR + TPR) % TPR;
                    const bool hasN = y > 0, hasS = y < ny - 1;
                    const int yN = hasN ? y - 1 : y, yS = hasS ? y + 1 : y;
                    int d = t - 2 * g, sd = d % R;
                    for (; g <= ghi; g += TPR) {
                        const DiffNb<T> a = load(sd, y, d - y, hasN, hasS, yN, yS);
                        ring[sd * ny + y] = diff_cell<T>(a.c, a.n, a.s, a.e, a.w, lambda, Ksq);
                        d -= 2 * TPR;
                        sd -= dstep;
                        if (sd < 0) sd += R;
                    }
                }
            if (nn > 0) {
                T *sd = slot(dn);
#pragma unroll
                for (int k = 0; k < kDiffPf; k++) {
                    if (k >= npf) break;
                    const int i = threadIdx.x + k * blockDim.x;
                    if (i < nn) sd[i] = pf[k];
                }
            }
            const int df = t - 2 * gc + 1;  // final for this group
            if (df >= 0 && df < D) {
                const T *sd = slot(df);
                for (int i = threadIdx.x; i < len(df); i += blockDim.x) U[cell(df, i)] = sd[i];
            }
            __syncthreads();
        }
        {
            const T *sd = slot(D - 1);
            for (int i = threadIdx.x; i < len(D - 1); i += blockDim.x) U[cell(D - 1, i)] = sd[i];
        }
        __syncthreads();
    }
}

// The row form with two rows per thread: rows (2r, 2r + 1) meet a diagonal d
// at adjacent positions of its slot, so one thread updates both cells of a
// sweep together: their centres, the W of the first (= N of the second) and
// the second's W, the first's E and S (= E of the second) and the second's S
// come from three 8-byte and two 4-byte shared-memory loads instead of ten,
// the two results go out as one 8-byte store, and the FP32 arithmetic of the
// pair runs as paired instructions (each the same IEEE operation as
// diff_cell's, so the results are bit-identical).  A pair whose second row
// or either cell is off the plane writes that position's old value back (the
// position belongs to no cell of the diagonal; only this thread writes it).
// A warp owns 64 rows and one of TPR sweep classes.  Slots are S >= ny + 1
// values (S even: the pairs' 8-byte accesses stay aligned).  Requires
// min(ny, nx) <= kDiffPf * blockDim.x, blockDim.x a multiple of 32 TPR and,
// FP32, blockDim.x <= 768.
template <typename T, int TPR>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 768 : 1024, sizeof(T) == 4 ? 2 : 1)
k_diffusion_pairs(T *u, int ny, int nx, int nxb, double lambda_d, double ksq_d, int niter,
                  int G, int R, int S)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T *ring = (T *)smraw;  // R slots of S >= ny + 1 values (S even)
    T *U = u + (size_t)blockIdx.x * ny * nx;
    const T lambda = (T)lambda_d, Ksq = (T)ksq_d;
    const int D = ny + nx - 1, L = min(ny, nx);
    auto y0 = [&](int d) { return max(0, d - (nx - 1)); };
    auto len = [&](int d) { return min(d, ny - 1) - y0(d) + 1; };
    auto slot = [&](int d) { return ring + (size_t)(d % R) * S + y0(d); };
    auto cell = [&](int d, int i) -> size_t {
        int a = y0(d);
        return (size_t)(a + i) * nx + (d - a - i);
    };
    using T2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cls = warp % TPR;
    const int pfirst = (warp / TPR) * 32 + lane, pstride = blockDim.x / TPR;
    const int dstep = (2 * TPR) % R;
    const int npairs = (ny + 1) >> 1;
    for (int s0 = 0; s0 < niter; s0 += G) {
        const int gc = min(G, niter - s0);
        const int nsteps = D + 2 * (gc - 1);
        for (int d = 0; d < 2 && d < D; d++) {
            T *sd = slot(d);
            for (int i = threadIdx.x; i < len(d); i += blockDim.x) sd[i] = U[cell(d, i)];
        }
        __syncthreads();
        for (int t = 0; t < nsteps; t++) {
            const int dn = t + 2;
            const int nn = dn < D ? len(dn) : 0;
            const int npf = (L + blockDim.x - 1) / blockDim.x;
            T pf[kDiffPf];
#pragma unroll
            for (int k = 0; k < kDiffPf; k++) {
                if (k >= npf) break;
                const int i = threadIdx.x + k * blockDim.x;
                pf[k] = i < nn ? U[cell(dn, i)] : T(0);
            }
            if (cls < gc)
                for (int pr = pfirst; pr < npairs && 2 * pr <= t; pr += pstride) {
                    const int y = 2 * pr;  // rows y, y + 1
                    // sweeps of this class with a cell in row y or y + 1:
                    // x = t - y - 2g in [0, nx] (row y + 1 has x - 1) and g < gc
                    const int ghi = min(gc - 1, (t - y) >> 1);
                    const int over = t - y - nx;  // x <= nx  <=>  g >= over / 2
                    const int glo = over > 0 ? (over + 1) >> 1 : 0;
                    int g = glo + ((cls - glo) % TPR + TPR) % TPR;
                    const bool hasN = y > 0, hasS1 = y + 1 < ny - 1;
                    const int yN = hasN ? y - 1 : y + 1;  // in-slot when clamped
                    const int yS = y + 2 < S ? y + 2 : y;
                    int d = t - 2 * g, sd = d % R;
                    for (; g <= ghi; g += TPR) {
                        const int x = d - y;  // row y + 1: x - 1
                        const int sm = sd == 0 ? R - 1 : sd - 1, sp = sd == R - 1 ? 0 : sd + 1;
                        T *rc = ring + sd * S;
                        const T *rm = ring + sm * S, *rp = ring + sp * S;
                        const T2 c = *reinterpret_cast<const T2 *>(rc + y);
                        const T2 m = *reinterpret_cast<const T2 *>(rm + y);  // W0 = N1, W1
                        const T2 q = *reinterpret_cast<const T2 *>(rp + y);  // E0, S0 = E1
                        const T mN = rm[yN], pS = rp[yS];
                        // row y: N = rm[y-1], W = rm[y], S = rp[y+1], E = rp[y]
                        // row y+1: N = rm[y], W = rm[y+1], S = rp[y+2], E = rp[y+1]
                        const int x1 = x - 1;
                        T n0 = hasN ? mN : c.x, w0 = x > 0 ? m.x : c.x, s0v = q.y;
                        T e0 = x == nxb - 1 ? c.x : (x + 1 < nx ? q.x : T(0));
                        if (y == ny - 1) s0v = c.x;  // last row (odd ny): S clamps to itself
                        T n1 = m.x, w1 = x1 > 0 ? m.y : c.y, s1 = hasS1 ? pS : c.y;
                        T e1 = x1 == nxb - 1 ? c.y : (x1 + 1 < nx ? q.y : T(0));
                        T u0, u1;
                        if constexpr (sizeof(T) == 4) {
                            auto f2 = [](float a, float b) { return make_float2(a, b); };
                            auto sub = [](float2 a, float2 b) {
                                return __fadd2_rn(a, make_float2(-b.x, -b.y));
                            };
                            const float2 cc = f2(c.x, c.y), k2 = f2(Ksq, Ksq);
                            const float2 gN = sub(f2(n0, n1), cc), gS = sub(f2(s0v, s1), cc),
                                         gE = sub(f2(e0, e1), cc), gW = sub(f2(w0, w1), cc);
                            auto coef = [&](float2 gg) {
                                const float2 dd = __ffma2_rn(gg, gg, k2);
                                return __fmul2_rn(k2, f2(rcp_approx(dd.x), rcp_approx(dd.y)));
                            };
                            float2 sum = __fmul2_rn(coef(gN), gN);
                            sum = __ffma2_rn(coef(gS), gS, sum);
                            sum = __ffma2_rn(coef(gE), gE, sum);
                            sum = __ffma2_rn(coef(gW), gW, sum);
                            const float2 uu = __ffma2_rn(f2(lambda, lambda), sum, cc);
                            u0 = uu.x;
                            u1 = uu.y;
                        } else {
                            u0 = diff_cell<T>(c.x, n0, s0v, e0, w0, lambda, Ksq);
                            u1 = diff_cell<T>(c.y, n1, s1, e1, w1, lambda, Ksq);
                        }
                        // a cell off the plane keeps its slot's old value
                        if (x > nx - 1) u0 = c.x;
                        if (x1 < 0 || y + 1 >= ny) u1 = c.y;
                        T2 o;
                        o.x = u0;
                        o.y = u1;
                        *reinterpret_cast<T2 *>(rc + y) = o;
                        d -= 2 * TPR;
                        sd -= dstep;
                        if (sd < 0) sd += R;
                    }
                }
            if (nn > 0) {
                T *sd = slot(dn);
#pragma unroll
                for (int k = 0; k < kDiffPf; k++) {
                    if (k >= npf) break;
                    const int i = threadIdx.x + k * blockDim.x;
                    if (i < nn) sd[i] = pf[k];
                }
            }
            const int df = t - 2 * gc + 1;
            if (df >= 0 && df < D) {
                const T *sd = slot(df);
                for (int i = threadIdx.x; i < len(df); i += blockDim.x) U[cell(df, i)] = sd[i];
            }
            __syncthreads();
        }
        {
            const T *sd = slot(D - 1);
            for (int i = threadIdx.x; i < len(D - 1); i += blockDim.x) U[cell(D - 1, i)] = sd[i];
        }
        __syncthreads();
    }
}

// The wavefront form: pairs (k_diffusion_pairs, the FP32 default), rows
// (k_diffusion_rows) or task tables (k_diffusion_ring, the FP64 default: the
// FP64 pipe bounds every form there and the tables form measured fastest);
// NUDIM_DIFFUSION=pairs|rows|tables selects one.  All give the same cells bit
// for bit.  Read at every launch (a captured graph keeps the form it was
// captured with).
enum DiffForm { DF_PAIRS, DF_ROWS, DF_TABLES };
template <typename T> static DiffForm diffusion_form()
{
    const char *e = getenv("NUDIM_DIFFUSION");
    if (e && !strcmp(e, "tables")) return DF_TABLES;
    if (e && !strcmp(e, "rows")) return DF_ROWS;
    if (e && !strcmp(e, "pairs")) return DF_PAIRS;
    return sizeof(T) == 8 ? DF_TABLES : DF_PAIRS;
}

template <typename T>
int diffusion_run(T *u, int nz, int ny, int nx, int nx_bound, float lambda, float kappa,
                  int niter, cudaStream_t st)
{
    if (niter <= 0 || nz <= 0) return NUDIM_OK;
    double ksq = (double)kappa * (double)kappa;
    int L = ny < nx ? ny : nx;
    int P = std::min(1024, (L + 31) & ~31);
    // FP32 on planes up to 512 wide: two CTAs per SM; otherwise one CTA with
    // up to 160 KB of ring
    bool two = sizeof(T) == 4 && P <= 512;
    const size_t budget = two ? ((size_t)108 << 10) : ((size_t)160 << 10);
    const DiffForm form = diffusion_form<T>();
    const int cap = sizeof(T) == 4 ? 768 : 1024;
    if (form == DF_PAIRS) {
        // two rows per thread: slots of S = ny + 1 rounded up to even values;
        // TPR sweep classes (a power of two) so that 64-row warps x classes
        // fill up to 768 (FP32, two CTAs per SM) or 1024 threads
        const int S = (ny + 2) & ~1, Pp = (((ny + 1) >> 1) + 31) & ~31;
        int G = (int)((budget / (sizeof(T) * (size_t)S) - 2) / 2);
        if (G > niter) G = niter;
        if (G > kDiffMaxG) G = kDiffMaxG;
        int tpr = 1;
        while (tpr < 8 && 2 * tpr * Pp <= cap && 2 * tpr <= G) tpr *= 2;
        const int threads = std::min(cap, tpr * Pp);
        if (G >= 1 && L <= kDiffPf * threads) {
            const int R = 2 * G + 2;
            const size_t smem = sizeof(T) * (size_t)R * S;
#define NUDIM_DIFF_PAIRS(TP)                                                                    \
    do {                                                                                        \
        NUDIM_CUDA(cudaFuncSetAttribute(k_diffusion_pairs<T, TP>,                               \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 160 << 10)); \
        k_diffusion_pairs<T, TP><<<nz, threads, smem, st>>>(u, ny, nx, nx_bound, (double)lambda, \
                                                             ksq, niter, G, R, S);              \
    } while (0)
            if (tpr == 8) NUDIM_DIFF_PAIRS(8);
            else if (tpr == 4) NUDIM_DIFF_PAIRS(4);
            else if (tpr == 2) NUDIM_DIFF_PAIRS(2);
            else NUDIM_DIFF_PAIRS(1);
#undef NUDIM_DIFF_PAIRS
            NUDIM_LAUNCH_CHECK();
            return NUDIM_OK;
        }
    }
    if (form == DF_ROWS) {
        // one row per thread: slots of ny values; TPR sweep classes so that
        // 32-row warps x classes fill up to 768 or 1024 threads
        int G = (int)((budget / (sizeof(T) * (size_t)ny) - 2) / 2);
        if (G > niter) G = niter;
        if (G > kDiffMaxG) G = kDiffMaxG;
        const int Py = (ny + 31) & ~31;
        int tpr = 1;
        while (tpr < 8 && 2 * tpr * Py <= cap && 2 * tpr <= G) tpr *= 2;
        const int threads = std::min(cap, tpr * Py);
        if (G >= 1 && L <= kDiffPf * threads) {
            const int R = 2 * G + 2;
            const size_t smem = sizeof(T) * (size_t)R * ny;
#define NUDIM_DIFF_ROWS(TP)                                                                     \
    do {                                                                                        \
        NUDIM_CUDA(cudaFuncSetAttribute(k_diffusion_rows<T, TP>,                                \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 160 << 10)); \
        k_diffusion_rows<T, TP><<<nz, threads, smem, st>>>(u, ny, nx, nx_bound, (double)lambda,  \
                                                            ksq, niter, G, R);                  \
    } while (0)
            if (tpr == 8) NUDIM_DIFF_ROWS(8);
            else if (tpr == 4) NUDIM_DIFF_ROWS(4);
            else if (tpr == 2) NUDIM_DIFF_ROWS(2);
            else NUDIM_DIFF_ROWS(1);
#undef NUDIM_DIFF_ROWS
            NUDIM_LAUNCH_CHECK();
            return NUDIM_OK;
        }
    }
    int threads = two ? 2 * P : 1024;
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
                            int, int, int, int, cudaStream_t, double *, double *);
template int tv_run<float>(float *, float *, double *, int, double *, int, int, int, float, int,
                           int, int, int, cudaStream_t, float *, float *);
template int diffusion_run<double>(double *, int, int, int, int, float, float, int, cudaStream_t);
template int diffusion_run<float>(float *, int, int, int, int, float, float, int, cudaStream_t);

}  // namespace nudim
