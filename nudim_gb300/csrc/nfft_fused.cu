// nfft_fused.cu -- the fused NFFT: the n0 x n1 oversampled grid never goes
// to HBM.  The uniform FFT factorises into a row pass and a column pass:
//
//   trafo   K1 row pass:   deconvolve + zero-pad each of the N0 nonzero rows,
//                          n1-point FFT in shared memory           -> H [N0][n1]
//           K2 column pass: load BC columns of H, n0-point FFTs in shared
//                          memory, Kaiser-Bessel interpolation partials of
//                          the nodes whose window meets these columns (half-
//                          warp per node, shuffle reduction)     -> partials
//           K3 combine:    f_j = sum of the node's partials (fixed order) +
//                          the CGNR / constraint epilogue
//   adjoint K4 column pass: spread the nodes into BC columns in shared memory
//                          (each warp owns a row band; nodes in ascending
//                          order; compensated FP32 sums), n0-point inverse
//                          FFTs, keep the N0 rows                 -> H'[N0][n1]
//           K5 row pass:   n1-point inverse FFT, crop to N1, deconvolve +
//                          epilogue (|z|^2 partials, p = z)
//
// No atomics: every output element has exactly one writer, and every sum
// has a fixed order, so results are deterministic.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "engine.cuh"

namespace nudim {

// ================================================================ smem FFT
template <typename T>
__device__ __forceinline__ cplx_t<T> cmul(cplx_t<T> a, cplx_t<T> b)
{
    return mkc<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// `cnt` FFTs of length n = 2^logn stored back to back in a; b is scratch.
// DIR = -1 forward (e^{-2 pi i}), +1 inverse; unnormalised.  Stockham
// autosort with radix-16 passes (a radix-8/4/2 pass last when 4 does not
// divide logn): each thread loads R elements at stride n/R, applies the
// twiddles e^{-2 pi i m k / (R Ns)} (table tw: e^{-2 pi i t/n}), does an
// R-point DFT in registers and stores R outputs at stride Ns.  Between
// passes the buffers hold element i at i + i/16, so the strided stores of
// the first passes meet distinct banks; the first pass reads and the last
// pass writes the plain layout.  Both buffers need fft_buf(cnt * n)
// elements.  All threads of the block call it; returns the buffer that
// holds the result (plain layout).
__host__ __device__ constexpr size_t fft_buf(size_t elems) { return elems + (elems >> 4); }
__device__ __forceinline__ int fft_pad(int i) { return i + (i >> 4); }

// e^{DIR 2 pi i k / 16}, k < 16, from cos(2 pi k / 16) for k = 0..4
template <typename T, int DIR> __device__ __forceinline__ cplx_t<T> w16(int k)
{
    constexpr double c[5] = {1.0, 0.92387953251128675613, 0.70710678118654752440,
                             0.38268343236508977173, 0.0};
    double cs, sn;
    int q = k & 3, h = k >> 2;  // k = 4h + q: rotate (cos, sin) of q by h quarter turns
    double cq = c[q], sq = c[4 - q];
    switch (h & 3) {
    case 0: cs = cq; sn = sq; break;
    case 1: cs = -sq; sn = cq; break;
    case 2: cs = -cq; sn = -sq; break;
    default: cs = sq; sn = -cq; break;
    }
    return mkc<T>((T)cs, (T)(DIR * sn));
}

template <typename T, int DIR>
__device__ __forceinline__ void dft2(cplx_t<T> &a0, cplx_t<T> &a1)
{
    cplx_t<T> t = a0;
    a0 = mkc<T>(t.x + a1.x, t.y + a1.y);
    a1 = mkc<T>(t.x - a1.x, t.y - a1.y);
}

template <typename T, int DIR>
__device__ __forceinline__ void dft4(cplx_t<T> &x0, cplx_t<T> &x1, cplx_t<T> &x2, cplx_t<T> &x3)
{
    using C = cplx_t<T>;
    C a0 = mkc<T>(x0.x + x2.x, x0.y + x2.y), a1 = mkc<T>(x0.x - x2.x, x0.y - x2.y);
    C a2 = mkc<T>(x1.x + x3.x, x1.y + x3.y), a3 = mkc<T>(x1.x - x3.x, x1.y - x3.y);
    x0 = mkc<T>(a0.x + a2.x, a0.y + a2.y);
    x2 = mkc<T>(a0.x - a2.x, a0.y - a2.y);
    // forward: X1 = a1 - i a3, X3 = a1 + i a3; inverse: the other way
    if (DIR < 0) {
        x1 = mkc<T>(a1.x + a3.y, a1.y - a3.x);
        x3 = mkc<T>(a1.x - a3.y, a1.y + a3.x);
    } else {
        x1 = mkc<T>(a1.x - a3.y, a1.y + a3.x);
        x3 = mkc<T>(a1.x + a3.y, a1.y - a3.x);
    }
}

// R-point DFT of a[0..R) in registers.  Output X[p] is left in a[out(p)]:
// R = 16 and 8 are split as R1 = 4 inner DFTs over m = R2 m1 + m2, the
// twiddles e^{DIR 2 pi i m2 p1 / R} and R2-point outer DFTs, X[p1 + 4 p2] in
// a[R2 p1 + p2].
template <int R> __device__ __forceinline__ constexpr int dft_out(int p)
{
    return R == 16 ? 4 * (p & 3) + (p >> 2) : R == 8 ? 2 * (p & 3) + (p >> 2) : p;
}

template <typename T, int DIR, int R> __device__ __forceinline__ void dft_regs(cplx_t<T> *a)
{
    if (R == 2) {
        dft2<T, DIR>(a[0], a[1]);
    } else if (R == 4) {
        dft4<T, DIR>(a[0], a[1], a[2], a[3]);
    } else if (R == 8) {
#pragma unroll
        for (int m2 = 0; m2 < 2; m2++) dft4<T, DIR>(a[m2], a[2 + m2], a[4 + m2], a[6 + m2]);
#pragma unroll
        for (int p1 = 1; p1 < 4; p1++) a[2 * p1 + 1] = cmul<T>(a[2 * p1 + 1], w16<T, DIR>(2 * p1));
#pragma unroll
        for (int p1 = 0; p1 < 4; p1++) dft2<T, DIR>(a[2 * p1], a[2 * p1 + 1]);
    } else {
#pragma unroll
        for (int m2 = 0; m2 < 4; m2++)
            dft4<T, DIR>(a[m2], a[4 + m2], a[8 + m2], a[12 + m2]);
#pragma unroll
        for (int p1 = 1; p1 < 4; p1++)
#pragma unroll
            for (int m2 = 1; m2 < 4; m2++)
                a[4 * p1 + m2] = cmul<T>(a[4 * p1 + m2], w16<T, DIR>(m2 * p1));
#pragma unroll
        for (int p1 = 0; p1 < 4; p1++)
            dft4<T, DIR>(a[4 * p1], a[4 * p1 + 1], a[4 * p1 + 2], a[4 * p1 + 3]);
    }
}

template <typename T, int DIR, int R, bool IN_PAD, bool OUT_PAD>
__device__ __forceinline__ void fft_pass(const cplx_t<T> *__restrict__ x, cplx_t<T> *__restrict__ y,
                                         int n, int lognR, int Ns, int cnt,
                                         const cplx_t<T> *__restrict__ tw)
{
    using C = cplx_t<T>;
    const int nR = 1 << lognR, step = n / (R * Ns);
    for (int q = threadIdx.x; q < cnt * nR; q += blockDim.x) {
        const int s = q >> lognR, j = q & (nR - 1), k = j & (Ns - 1);
        const int base = s * n;
        C a[R];
#pragma unroll
        for (int m = 0; m < R; m++) {
            int i = base + j + m * nR;
            a[m] = x[IN_PAD ? fft_pad(i) : i];
        }
        if (Ns > 1) {
            const int ks = k * step;
#pragma unroll
            for (int m = 1; m < R; m++) {
                C w = tw[m * ks];
                if (DIR > 0) w.y = -w.y;
                a[m] = cmul<T>(a[m], w);
            }
        }
        dft_regs<T, DIR, R>(a);
        const int ob = base + (j - k) * R + k;
#pragma unroll
        for (int p = 0; p < R; p++) {
            int i = ob + p * Ns;
            y[OUT_PAD ? fft_pad(i) : i] = a[dft_out<R>(p)];
        }
    }
}

template <typename T, int DIR, int R>
__device__ __forceinline__ void fft_pass_sel(const cplx_t<T> *x, cplx_t<T> *y, int n, int lognR,
                                             int Ns, int cnt, const cplx_t<T> *tw, bool first,
                                             bool last)
{
    if (first && last) fft_pass<T, DIR, R, false, false>(x, y, n, lognR, Ns, cnt, tw);
    else if (first) fft_pass<T, DIR, R, false, true>(x, y, n, lognR, Ns, cnt, tw);
    else if (last) fft_pass<T, DIR, R, true, false>(x, y, n, lognR, Ns, cnt, tw);
    else fft_pass<T, DIR, R, true, true>(x, y, n, lognR, Ns, cnt, tw);
}

template <typename T, int DIR>
__device__ cplx_t<T> *block_fft(cplx_t<T> *a, cplx_t<T> *b, int n, int logn, int cnt,
                                const cplx_t<T> *__restrict__ tw)
{
    const int npass = (logn + 3) >> 2;
    int rem = logn, Ns = 1;
    for (int t = 0; t < npass; t++) {
        const int lr = rem < 4 ? rem : 4;
        const bool first = t == 0, last = t == npass - 1;
        const int lognR = logn - lr;
        switch (lr) {
        case 4: fft_pass_sel<T, DIR, 16>(a, b, n, lognR, Ns, cnt, tw, first, last); break;
        case 3: fft_pass_sel<T, DIR, 8>(a, b, n, lognR, Ns, cnt, tw, first, last); break;
        case 2: fft_pass_sel<T, DIR, 4>(a, b, n, lognR, Ns, cnt, tw, first, last); break;
        default: fft_pass_sel<T, DIR, 2>(a, b, n, lognR, Ns, cnt, tw, first, last); break;
        }
        rem -= lr;
        Ns <<= lr;
        cplx_t<T> *t2 = a;
        a = b;
        b = t2;
        __syncthreads();
    }
    return a;
}


// ================================================================ four-step register FFT
// n = R1 x R2 points with one shared-memory exchange: input index l = j +
// R2 m (j < R2, m < R1), pass 1 an R1-point DFT over m per j (registers),
// twiddle W_n^{j k1}, exchange, pass 2 an R2-point DFT over j per k1, output
// index k = k1 + R1 k2 (the classical four-step factorisation of the DFT).
// R = 32 DFTs in registers split as two 16-point DFTs (dft_regs<16>) and a
// radix-2 step with the twiddles W_32^p.
template <typename T, int DIR> __device__ __forceinline__ cplx_t<T> w32(int p)
{
    // cos(2 pi p / 32), p = 0..8
    constexpr double c[9] = {1.0,
                             0.98078528040323044913,
                             0.92387953251128675613,
                             0.83146961230254523708,
                             0.70710678118654752440,
                             0.55557023301960222474,
                             0.38268343236508977173,
                             0.19509032201612826785,
                             0.0};
    const int q = p & 7, h = p >> 3;  // p = 8h + q: rotate by h quarter turns
    double cs, sn;
    const double cq = c[q], sq = c[8 - q];
    switch (h & 3) {
    case 0: cs = cq; sn = sq; break;
    case 1: cs = -sq; sn = cq; break;
    case 2: cs = -cq; sn = -sq; break;
    default: cs = sq; sn = -cq; break;
    }
    return mkc<T>((T)cs, (T)(DIR * sn));
}

// W_24^p = e^{DIR 2 pi i p / 24}, p = 0..23
template <typename T, int DIR> __device__ __forceinline__ cplx_t<T> w24(int p)
{
    // cos(2 pi q / 24), q = 0..6
    constexpr double c[7] = {1.0,
                             0.96592582628906828675,
                             0.86602540378443864676,
                             0.70710678118654752440,
                             0.5,
                             0.25881904510252076235,
                             0.0};
    const int q = p % 6, h = p / 6;  // p = 6h + q: rotate by h quarter turns
    double cs, sn;
    const double cq = c[q], sq = c[6 - q];
    switch (h & 3) {
    case 0: cs = cq; sn = sq; break;
    case 1: cs = -sq; sn = cq; break;
    case 2: cs = -cq; sn = -sq; break;
    default: cs = sq; sn = -cq; break;
    }
    return mkc<T>((T)cs, (T)(DIR * sn));
}

// R-point DFT (R = 16, 24 or 32) of a[0..R) in registers; X[p] is left in
// a[fs_out<R>(p)].  R = 24: three 8-point DFTs over a[3u + v], the twiddles
// W_24^{v p8} and 3-point DFTs over v, X[p8 + 8q] in a[3 p8 + q].
template <int R> __device__ __forceinline__ constexpr int fs_out(int p)
{
    return R == 16   ? dft_out<16>(p)
           : R == 24 ? 3 * (p & 7) + (p >> 3)
                     : (p < 16 ? 2 * dft_out<16>(p) : 2 * dft_out<16>(p - 16) + 1);
}

template <typename T, int DIR, int R> __device__ __forceinline__ void fs_dft(cplx_t<T> *a)
{
    using C = cplx_t<T>;
    if constexpr (R == 16) {
        dft_regs<T, DIR, 16>(a);
    } else if constexpr (R == 24) {
        C e[3][8];
#pragma unroll
        for (int v = 0; v < 3; v++)
#pragma unroll
            for (int u = 0; u < 8; u++) e[v][u] = a[3 * u + v];
#pragma unroll
        for (int v = 0; v < 3; v++) dft_regs<T, DIR, 8>(e[v]);
        // X[p8 + 8q] = sum_v (W_24^{v p8} E_v[p8]) W_3^{v q}
        const T h3 = (T)0.86602540378443864676;  // sqrt(3) / 2
#pragma unroll
        for (int p8 = 0; p8 < 8; p8++) {
            const C x0 = e[0][dft_out<8>(p8)];
            C x1 = e[1][dft_out<8>(p8)], x2 = e[2][dft_out<8>(p8)];
            if (p8) {
                x1 = cmul<T>(x1, w24<T, DIR>(p8));
                x2 = cmul<T>(x2, w24<T, DIR>(2 * p8));
            }
            const C sm = mkc<T>(x1.x + x2.x, x1.y + x2.y), df = mkc<T>(x1.x - x2.x, x1.y - x2.y);
            const C mid = mkc<T>(x0.x - (T)0.5 * sm.x, x0.y - (T)0.5 * sm.y);
            // DIR i (sqrt(3)/2) (x1 - x2)
            const C rot = mkc<T>(-(T)DIR * h3 * df.y, (T)DIR * h3 * df.x);
            a[3 * p8] = mkc<T>(x0.x + sm.x, x0.y + sm.y);
            a[3 * p8 + 1] = mkc<T>(mid.x + rot.x, mid.y + rot.y);
            a[3 * p8 + 2] = mkc<T>(mid.x - rot.x, mid.y - rot.y);
        }
    } else {
        C e[16], o[16];
#pragma unroll
        for (int u = 0; u < 16; u++) {
            e[u] = a[2 * u];
            o[u] = a[2 * u + 1];
        }
        dft_regs<T, DIR, 16>(e);
        dft_regs<T, DIR, 16>(o);
        // X[p] = E[p] + W32^p O[p], X[p + 16] = E[p] - W32^p O[p]
#pragma unroll
        for (int p = 0; p < 16; p++) {
            const C ev = e[dft_out<16>(p)];
            C ov = o[dft_out<16>(p)];
            if (p) ov = cmul<T>(ov, w32<T, DIR>(p));
            a[2 * dft_out<16>(p)] = mkc<T>(ev.x + ov.x, ev.y + ov.y);
            a[2 * dft_out<16>(p) + 1] = mkc<T>(ev.x - ov.x, ev.y - ov.y);
        }
    }
}

template <int R1, int R2> __host__ __device__ constexpr int fs_col_stride()
{
    // R1 x (R2 + 1) rounded up to 4 mod 16 elements
    return ((R1 * (R2 + 1) + 11) / 16) * 16 + 4;
}

// ================================================================ K1 row pass (trafo)
template <typename T, int MODE>
__global__ void __launch_bounds__(256)
k_rowfft(const void *__restrict__ src, size_t src_stride, int N0, int N1, int n1, int logn1,
         int kRows, const T *__restrict__ c0, const T *__restrict__ c1,
         const cplx_t<T> *__restrict__ tw1, int plane0, cplx_t<T> *__restrict__ H,
         cplx_t<T> *__restrict__ f_init, size_t f_stride)
{
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *A = (C *)smraw, *B = A + fft_buf((size_t)kRows * n1);
    int b = blockIdx.y, gb = plane0 + b, a0 = blockIdx.x * kRows;
    int nr = min(kRows, N0 - a0);
    // eight elements per thread in flight before the shared-memory stores
    constexpr int U = 8;
    const int total = nr * n1;
    for (int base = threadIdx.x; base < total; base += U * blockDim.x) {
        C v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int idx = base + u * blockDim.x;
            const int r = idx / n1, l1 = idx - r * n1;
            const int k1 = l1 < n1 / 2 ? l1 : l1 - n1;
            v[u] = mkc<T>(0, 0);
            if (idx < total && k1 >= -N1 / 2 && k1 < N1 / 2) {
                int a = a0 + r, c = k1 + N1 / 2;
                size_t o = (size_t)gb * src_stride + (size_t)a * N1 + c;
                C s;
                if (MODE == PM_COMPLEX) {
                    s = ((const C *)src)[o];
                } else {
                    s = mkc<T>(((const T *)src)[o], T(0));
                    f_init[(size_t)gb * f_stride + (size_t)a * N1 + c] = s;
                }
                T sc = c0[a] * c1[c];
                v[u] = mkc<T>(s.x * sc, s.y * sc);
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int idx = base + u * blockDim.x;
            if (idx < total) A[idx] = v[u];
        }
    }
    __syncthreads();
    C *R = block_fft<T, -1>(A, B, n1, logn1, nr, tw1);
    C *Hb = H + ((size_t)b * N0 + a0) * n1;
    for (int idx = threadIdx.x; idx < nr * n1; idx += blockDim.x) Hb[idx] = R[idx];
}

// ================================================================ K2 column pass + interpolation
// warps per trafo column-block CTA (register room for the radix-16 FFT passes
// and the row weights)
template <typename T> __host__ __device__ constexpr int col_warps() { return 8; }

// Shared memory: two BC x n0 complex buffers (FFT).  After the column FFTs
// each lane takes one (node, block) entry of the block's list and sums the
// node's window over the block's columns: for each of the cnt columns
// inside the window, the 14-row column sum weighted by the row weights,
// then weighted by the column's weight.  Entry records are structures of
// arrays (coalesced across the lanes); rows are read in 16-byte aligned
// pairs (FP32) against 16 row weights pre-shifted to the even first row.
// The list holds entries with equal cnt side by side, so the lanes of a
// warp run loops of equal length.
#ifndef NUDIM_COL_MINB
#define NUDIM_COL_MINB 3  // FP32 CTAs per SM the register allocation aims for
#endif
template <typename T>
__global__ void __launch_bounds__(32 * col_warps<T>(), sizeof(T) == 4 ? NUDIM_COL_MINB : 1)
k_colfft_interp(const cplx_t<T> *__restrict__ H, int N0, int n0, int logn0, int n1, int BC,
                const cplx_t<T> *__restrict__ tw0, const int *__restrict__ blk_off,
                const int *__restrict__ ent, const int *__restrict__ e_rb,
                const int *__restrict__ e_cc, const T *__restrict__ e_qa,
                const T *__restrict__ e_q1, int nE, int M, int smax,
                cplx_t<T> *__restrict__ part)
{
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *A = (C *)smraw, *B = A + fft_buf((size_t)BC * n0);
    int cb = blockIdx.x, b = blockIdx.y;
    const C *Hb = H + (size_t)b * N0 * n1 + (size_t)cb * BC;
    // rows a of H land at l0 = (a - N0/2) mod n0; the other rows are zero.
    // Eight loads per thread in flight before the shared-memory stores.
    {
        constexpr int U = 8;
        const int total = n0 * BC;
        for (int base = threadIdx.x; base < total; base += U * blockDim.x) {
            C v[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int idx = base + u * blockDim.x;
                const int l0 = idx / BC, c = idx - l0 * BC;
                const int k0 = l0 < n0 / 2 ? l0 : l0 - n0;
                v[u] = mkc<T>(0, 0);
                if (idx < total && k0 >= -N0 / 2 && k0 < N0 / 2)
                    v[u] = Hb[(size_t)(k0 + N0 / 2) * n1 + c];
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int idx = base + u * blockDim.x;
                const int l0 = idx / BC, c = idx - l0 * BC;
                if (idx < total) A[(size_t)c * n0 + l0] = v[u];
            }
        }
    }
    __syncthreads();
    const C *G = block_fft<T, -1>(A, B, n0, logn0, BC, tw0);
    const int beg = blk_off[cb], end = blk_off[cb + 1];
    const int m0 = n0 - 1;
    for (int e = beg + threadIdx.x; e < end; e += blockDim.x) {
        const int js = ent[e], rb = e_rb[e], ccn = e_cc[e];
        const int cl0 = ccn & 255, cnt = (ccn >> 8) & 255;
        T qa[16];
#pragma unroll
        for (int i = 0; i < 16; i++) qa[i] = e_qa[(size_t)i * nE + e];
        T ar = 0, ai = 0;
        for (int q = 0; q < cnt; q++) {
            const C *gp = G + (size_t)((cl0 + q) & (BC - 1)) * n0;
            T sr = 0, si = 0;
            if constexpr (sizeof(T) == 4) {
                // FP32 form: one paired FMA per row, (re, im) += q * g
                float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    float4 pr = *(const float4 *)(gp + ((rb + 2 * i) & m0));
                    s2 = __ffma2_rn(make_float2(qa[2 * i], qa[2 * i]), make_float2(pr.x, pr.y), s2);
                    s2 = __ffma2_rn(make_float2(qa[2 * i + 1], qa[2 * i + 1]),
                                    make_float2(pr.z, pr.w), s2);
                }
                sr = s2.x;
                si = s2.y;
            } else {
                // FP64: the window's 14 rows only (the 16-row pairs are an
                // FP32 load shape; every FMA counts on the FP64 pipe)
                const int odd = ccn >> 16;
#pragma unroll
                for (int i = 0; i < 14; i++) {
                    const T w = odd ? qa[i + 1] : qa[i];
                    C g = gp[(rb + odd + i) & m0];
                    sr += w * g.x;
                    si += w * g.y;
                }
            }
            T w = e_q1[(size_t)q * nE + e];
            ar += w * sr;
            ai += w * si;
        }
        part[((size_t)b * smax + (js & 7)) * M + (js >> 3)] = mkc<T>(ar, ai);
    }
}

// ================================================================ K2' column pass, four-step
// k_colfft_interp with the column FFTs as four-step register FFTs (n0 =
// R1 x R2, BC = 4): the first 4 R2 threads read the block's N0 nonzero rows
// of H straight into pass 1's registers (a warp reads 8 rows x 4 columns
// per step), exchange through shared memory, and pass 2 writes the columns
// to Gs (column stride n0 + 8: the four columns' stores meet distinct
// banks); then every thread interpolates as in k_colfft_interp.
template <typename T, int R1, int R2>
__global__ void __launch_bounds__(32 * col_warps<T>(), sizeof(T) == 4 ? NUDIM_COL_MINB : 1)
k_colfft_interp_fs(const cplx_t<T> *__restrict__ H, int N0, int n1,
                   const cplx_t<T> *__restrict__ tw0, const int *__restrict__ blk_off,
                   const int *__restrict__ ent, const int *__restrict__ e_rb,
                   const int *__restrict__ e_cc, const T *__restrict__ e_qa,
                   const T *__restrict__ e_q1, int nE, int M, int smax,
                   cplx_t<T> *__restrict__ part)
{
    using C = cplx_t<T>;
    constexpr int n0 = R1 * R2, BC = 4, GS = n0 + 8, CS = fs_col_stride<R1, R2>();
    extern __shared__ __align__(16) unsigned char smraw[];
    C *Gs = (C *)smraw, *S = Gs + BC * GS;
    const int cb = blockIdx.x, b = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool fft = threadIdx.x < 4 * R2;
    const int c = lane & 3, j = warp * 8 + (lane >> 2);
    if (fft) {
        const C *Hb = H + (size_t)b * N0 * n1 + (size_t)cb * BC + c;
        C x[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
            const int l0 = j + R2 * m;
            const int a = (l0 < n0 / 2 ? l0 : l0 - n0) + N0 / 2;
            x[m] = (a >= 0 && a < N0) ? Hb[(size_t)a * n1] : mkc<T>(0, 0);
        }
        fs_dft<T, -1, R1>(x);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            C v = x[fs_out<R1>(k1)];
            if (k1) v = cmul<T>(v, tw0[j * k1]);
            S[c * CS + k1 * (R2 + 1) + j] = v;
        }
    }
    __syncthreads();
    if (fft) {
        for (int k1 = j; k1 < R1; k1 += R2) {
            C y[R2];
#pragma unroll
            for (int jj = 0; jj < R2; jj++) y[jj] = S[c * CS + k1 * (R2 + 1) + jj];
            fs_dft<T, -1, R2>(y);
#pragma unroll
            for (int k2 = 0; k2 < R2; k2++) Gs[c * GS + k1 + R1 * k2] = y[fs_out<R2>(k2)];
        }
    }
    __syncthreads();
    const int beg = blk_off[cb], end = blk_off[cb + 1];
    const int m0 = n0 - 1;
    for (int e = beg + threadIdx.x; e < end; e += blockDim.x) {
        const int js = ent[e], rb = e_rb[e], ccn = e_cc[e];
        const int cl0 = ccn & 255, cnt = (ccn >> 8) & 255;
        T qa[16];
#pragma unroll
        for (int i = 0; i < 16; i++) qa[i] = e_qa[(size_t)i * nE + e];
        T ar = 0, ai = 0;
        for (int q = 0; q < cnt; q++) {
            const C *gp = Gs + (size_t)((cl0 + q) & (BC - 1)) * GS;
            T sr = 0, si = 0;
            if constexpr (sizeof(T) == 4) {
                float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    float4 pr = *(const float4 *)(gp + ((rb + 2 * i) & m0));
                    s2 = __ffma2_rn(make_float2(qa[2 * i], qa[2 * i]), make_float2(pr.x, pr.y), s2);
                    s2 = __ffma2_rn(make_float2(qa[2 * i + 1], qa[2 * i + 1]),
                                    make_float2(pr.z, pr.w), s2);
                }
                sr = s2.x;
                si = s2.y;
            } else {
                // FP64: the window's 14 rows only (the 16-row pairs are an
                // FP32 load shape; every FMA counts on the FP64 pipe)
                const int odd = ccn >> 16;
#pragma unroll
                for (int i = 0; i < 14; i++) {
                    const T w = odd ? qa[i + 1] : qa[i];
                    C g = gp[(rb + odd + i) & m0];
                    sr += w * g.x;
                    si += w * g.y;
                }
            }
            T w = e_q1[(size_t)q * nE + e];
            ar += w * sr;
            ai += w * si;
        }
        part[((size_t)b * smax + (js & 7)) * M + (js >> 3)] = mkc<T>(ar, ai);
    }
}

// ================================================================ K2'' column pass, two planes
// The FP32 trafo column pass for two Z-planes per CTA (n0 = R1 x R2, BC =
// 4): 128 threads run each plane's four column FFTs (all 256 busy), each
// plane's exchange goes through its own column buffer (pass 1 writes the
// twiddled rows there, a barrier, pass 2 reads them into registers, a
// barrier, pass 2 writes the transformed columns over them: one 4 x GS
// buffer per plane, GS = 4 mod 16 so neither pass meets a bank twice), and
// each thread then interpolates its (node, block) entries for both planes
// with one read of the entry's record: the record loads -- the column
// pass's long-latency reads -- are shared by two planes.
template <int R1, int R2> __host__ __device__ constexpr int fs2_gs()
{
    // at least R1 x (R2 + 1) (the exchange) and R1 R2 (the column), 4 mod 16
    return ((R1 * (R2 + 1) + 11) / 16) * 16 + 4;
}

template <int R1, int R2>
__global__ void __launch_bounds__(256, 3)
k_colfft_interp_fs2(const float2 *__restrict__ H, int N0, int n1, int nb_planes,
                    const float2 *__restrict__ tw0, const int *__restrict__ blk_off,
                    const int *__restrict__ ent, const int *__restrict__ e_rb,
                    const int *__restrict__ e_cc, const float *__restrict__ e_qa,
                    const float *__restrict__ e_q1, int nE, int M, int smax,
                    float2 *__restrict__ part)
{
    using C = float2;
    constexpr int n0 = R1 * R2, BC = 4, GS = fs2_gs<R1, R2>();
    extern __shared__ __align__(16) unsigned char smraw[];
    C *Gs = (C *)smraw;  // [plane 0..1][column][GS]
    const int cb = blockIdx.x, pb = blockIdx.y * 2;
    const bool two = pb + 1 < nb_planes;
    const int pp = threadIdx.x >> 7, t = threadIdx.x & 127;
    const int lane = t & 31, warp = t >> 5;
    const int c = lane & 3, j = warp * 8 + (lane >> 2);
    const bool fft = t < 4 * R2 && (pp == 0 || two);
    C *Gp = Gs + (size_t)pp * BC * GS;
    C y[R2];
    if (fft) {
        const C *Hb = H + (size_t)(pb + pp) * N0 * n1 + (size_t)cb * BC + c;
        C x[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
            const int l0 = j + R2 * m;
            const int a = (l0 < n0 / 2 ? l0 : l0 - n0) + N0 / 2;
            x[m] = (a >= 0 && a < N0) ? Hb[(size_t)a * n1] : make_float2(0.f, 0.f);
        }
        fs_dft<float, -1, R1>(x);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            C v = x[fs_out<R1>(k1)];
            if (k1) v = cmul<float>(v, tw0[j * k1]);
            Gp[c * GS + k1 * (R2 + 1) + j] = v;
        }
    }
    __syncthreads();
    // pass 2 (R1 / R2 columns of the exchange per thread; R1 == R2 here or
    // R1 = 2 R2): read them all before any thread overwrites the buffer
    constexpr int NK = R1 / R2;
    C yy[NK][R2];
    if (fft) {
#pragma unroll
        for (int q = 0; q < NK; q++) {
            const int k1 = j + q * R2;
#pragma unroll
            for (int jj = 0; jj < R2; jj++) yy[q][jj] = Gp[c * GS + k1 * (R2 + 1) + jj];
        }
    }
    __syncthreads();
    if (fft) {
#pragma unroll
        for (int q = 0; q < NK; q++) {
            const int k1 = j + q * R2;
#pragma unroll
            for (int jj = 0; jj < R2; jj++) y[jj] = yy[q][jj];
            fs_dft<float, -1, R2>(y);
#pragma unroll
            for (int k2 = 0; k2 < R2; k2++) Gp[c * GS + k1 + R1 * k2] = y[fs_out<R2>(k2)];
        }
    }
    __syncthreads();
    const int beg = blk_off[cb], end = blk_off[cb + 1];
    const int m0 = n0 - 1;
    for (int e = beg + threadIdx.x; e < end; e += blockDim.x) {
        const int js = ent[e], rb = e_rb[e], ccn = e_cc[e];
        const int cl0 = ccn & 255, cnt = (ccn >> 8) & 255;
        float qa[16];
#pragma unroll
        for (int i = 0; i < 16; i++) qa[i] = e_qa[(size_t)i * nE + e];
        float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
        for (int q = 0; q < cnt; q++) {
            const int col = (cl0 + q) & (BC - 1);
            const C *g0 = Gs + (size_t)col * GS, *g1 = g0 + BC * GS;
            float2 s0 = make_float2(0.f, 0.f), s1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int r = (rb + 2 * i) & m0;
                const float4 p0 = *(const float4 *)(g0 + r);
                const float4 p1 = *(const float4 *)(g1 + r);
                const float2 qa0 = make_float2(qa[2 * i], qa[2 * i]);
                const float2 qa1 = make_float2(qa[2 * i + 1], qa[2 * i + 1]);
                s0 = __ffma2_rn(qa0, make_float2(p0.x, p0.y), s0);
                s0 = __ffma2_rn(qa1, make_float2(p0.z, p0.w), s0);
                s1 = __ffma2_rn(qa0, make_float2(p1.x, p1.y), s1);
                s1 = __ffma2_rn(qa1, make_float2(p1.z, p1.w), s1);
            }
            const float w = e_q1[(size_t)q * nE + e];
            const float2 ww = make_float2(w, w);
            acc0 = __ffma2_rn(ww, s0, acc0);
            acc1 = __ffma2_rn(ww, s1, acc1);
        }
        part[((size_t)pb * smax + (js & 7)) * M + (js >> 3)] = acc0;
        if (two) part[((size_t)(pb + 1) * smax + (js & 7)) * M + (js >> 3)] = acc1;
    }
}

// ================================================================ K2 column pass, 8-column blocks
// The FP32 trafo column pass on blocks of 8 columns (n0 = R1 x R2): a
// node's 14 window columns meet 2 or 3 blocks instead of 4 or 5, so there
// are fewer (node, block) entries -- fewer record loads and partial sums --
// and more columns per entry.  256 threads run the 8 column FFTs (a warp
// reads 4 rows x 8 columns per step), the column buffer (stride GS = 2 mod
// 16) doubles as the exchange; then the interpolation as in
// k_colfft_interp.
template <int R1, int R2> __host__ __device__ constexpr int fs8_gs()
{
    return ((R1 * (R2 + 1) + 13) / 16) * 16 + 2;
}

template <int R1, int R2>
__global__ void __launch_bounds__(256, 3)
k_colfft_interp_fs8(const float2 *__restrict__ H, int N0, int n1,
                    const float2 *__restrict__ tw0, const int *__restrict__ blk_off,
                    const int *__restrict__ ent, const int *__restrict__ e_rb,
                    const int *__restrict__ e_cc, const float *__restrict__ e_qa,
                    const float *__restrict__ e_q1, int nE, int M, int smax,
                    float2 *__restrict__ part)
{
    using C = float2;
    constexpr int n0 = R1 * R2, BC = 8, GS = fs8_gs<R1, R2>();
    extern __shared__ __align__(16) unsigned char smraw[];
    C *Gs = (C *)smraw;  // [column][GS]
    const int cb = blockIdx.x, b = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = lane & 7, j = warp * 4 + (lane >> 3);
    const bool fft = j < R2;
    if (fft) {
        const C *Hb = H + (size_t)b * N0 * n1 + (size_t)cb * BC + c;
        C x[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
            const int l0 = j + R2 * m;
            const int a = (l0 < n0 / 2 ? l0 : l0 - n0) + N0 / 2;
            x[m] = (a >= 0 && a < N0) ? Hb[(size_t)a * n1] : make_float2(0.f, 0.f);
        }
        fs_dft<float, -1, R1>(x);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            C v = x[fs_out<R1>(k1)];
            if (k1) v = cmul<float>(v, tw0[j * k1]);
            Gs[c * GS + k1 * (R2 + 1) + j] = v;
        }
    }
    __syncthreads();
    constexpr int NK = R1 / R2;
    C yy[NK][R2];
    if (fft) {
#pragma unroll
        for (int q = 0; q < NK; q++) {
            const int k1 = j + q * R2;
#pragma unroll
            for (int jj = 0; jj < R2; jj++) yy[q][jj] = Gs[c * GS + k1 * (R2 + 1) + jj];
        }
    }
    __syncthreads();
    if (fft) {
#pragma unroll
        for (int q = 0; q < NK; q++) {
            const int k1 = j + q * R2;
            fs_dft<float, -1, R2>(yy[q]);
#pragma unroll
            for (int k2 = 0; k2 < R2; k2++) Gs[c * GS + k1 + R1 * k2] = yy[q][fs_out<R2>(k2)];
        }
    }
    __syncthreads();
    const int beg = blk_off[cb], end = blk_off[cb + 1];
    const int m0 = n0 - 1;
    for (int e = beg + threadIdx.x; e < end; e += blockDim.x) {
        const int js = ent[e], rb = e_rb[e], ccn = e_cc[e];
        const int cl0 = ccn & 255, cnt = (ccn >> 8) & 255;
        float qa[16];
#pragma unroll
        for (int i = 0; i < 16; i++) qa[i] = e_qa[(size_t)i * nE + e];
        float2 acc = make_float2(0.f, 0.f);
        for (int q = 0; q < cnt; q++) {
            const C *gp = Gs + (size_t)((cl0 + q) & (BC - 1)) * GS;
            float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const float4 pr = *(const float4 *)(gp + ((rb + 2 * i) & m0));
                s2 = __ffma2_rn(make_float2(qa[2 * i], qa[2 * i]), make_float2(pr.x, pr.y), s2);
                s2 = __ffma2_rn(make_float2(qa[2 * i + 1], qa[2 * i + 1]), make_float2(pr.z, pr.w),
                                s2);
            }
            const float w = e_q1[(size_t)q * nE + e];
            acc = __ffma2_rn(make_float2(w, w), s2, acc);
        }
        part[((size_t)b * smax + (js & 7)) * M + (js >> 3)] = acc;
    }
}

// ================================================================ K3 combine + epilogue
template <typename T, int MODE>
__global__ void __launch_bounds__(256)
k_combine(const cplx_t<T> *__restrict__ part, const unsigned char *__restrict__ nslots, int M,
          int smax, int plane0, InterpArgs<T> a)
{
    using C = cplx_t<T>;
    __shared__ double sh[32];
    int b = blockIdx.y, gb = plane0 + b;
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    T s0 = 0, s1 = 0;
    if (j < M) {
        // the node's partials (at most 8 slots) loaded together, summed in
        // slot order
        const int ns = nslots[j];
        C v[8];
        v[0] = part[((size_t)b * smax) * M + j];
#pragma unroll
        for (int s = 1; s < 8; s++)
            if (s < ns) v[s] = part[((size_t)b * smax + s) * M + j];
        C f = v[0];
#pragma unroll
        for (int s = 1; s < 8; s++)
            if (s < ns) {
                f.x += v[s].x;
                f.y += v[s].y;
            }
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
        } else {
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
            if (threadIdx.x == 0) a.part[(size_t)gb * a.part_stride + gridDim.x + blockIdx.x] = v1;
        }
    }
}

// Kahan-compensated sum of complex FP32 values with paired instructions:
// y = v - c, t = s + y, c = (t - s) - y, s = t (the subtractions as fused
// multiply-adds by -1, exact before their single rounding); the total is
// s - c.
struct Kahan2 {
    float2 s, c;
    __device__ __forceinline__ void init()
    {
        s = make_float2(0.f, 0.f);
        c = make_float2(0.f, 0.f);
    }
    __device__ __forceinline__ void add(float2 v)
    {
        const float2 m1 = make_float2(-1.f, -1.f);
        const float2 y = __ffma2_rn(m1, c, v);
        const float2 t = __fadd2_rn(s, y);
        c = __ffma2_rn(m1, y, __ffma2_rn(m1, s, t));
        s = t;
    }
    __device__ __forceinline__ float2 value() const
    {
        return __ffma2_rn(make_float2(-1.f, -1.f), c, s);
    }
};

// ================================================================ K4a spreading gather
// The adjoint's spreading as a gather into the oversampled grid G of a chunk
// of planes.  The grid is cut into tiles of R = 32 / BC rows x BC columns
// (one grid point per warp lane); each tile has the ascending list of the
// nodes whose window meets it, every entry carrying the tile's R row and BC
// column window weights (zero outside the window).  A warp takes one tile
// for P planes at a time and walks its list in chunks of 32 entries: lane l
// stages entry l's weights and its node's P (weighted) values in the warp's
// shared-memory stage, then every lane sums, for its grid point and each
// plane, q0(row) q1(col) f over the chunk -- one paired FMA per plane and
// entry in FP32.  FP32: plain sums within a chunk, Kahan-compensated across
// chunks; FP64: fused multiply-adds in ascending node order.  The tile's 32 points of each plane are one
// contiguous 256-byte (FP32) store: G is laid out column block by column
// block, [plane][block][row][column in block], which is also the order the
// column IFFT reads.  The work units are ranges of at most kGatherMaxEntries
// entries of a tile's list (the lists near the polar grid's centre run to
// over a thousand entries; a whole list per warp would make the longest one
// the kernel's critical path): a tile's first range writes G, its later
// ranges write partial sums that k_spread_fixup adds in range order.  Units
// come longest first; a CTA takes kGatherUnitsPerCta consecutive ones and
// its warps share them out through a shared counter.  No grid point has two
// writers and every sum has a fixed order: the results are deterministic.
constexpr int kGatherWarps = 8;
constexpr int kGatherUnitsPerCta = 16;
constexpr int kGatherMaxEntries = 128;

// node values of a stage: row stride in complex elements (padded so the
// lanes' 16-byte staging stores meet distinct banks)
template <int P> __host__ __device__ constexpr int gather_fs_stride() { return P == 1 ? 1 : P + 2; }
template <typename T, int P> __host__ __device__ constexpr size_t gather_stage_bytes(int W)
{
    return 32 * ((size_t)W * sizeof(T) + (size_t)gather_fs_stride<P>() * sizeof(cplx_t<T>));
}

template <typename T, bool WEIGHTED, int P>
__global__ void __launch_bounds__(32 * kGatherWarps, 3)
k_spread_gather(SpreadArgs<T> sa, const int4 *__restrict__ units, int nunits,
                const int *__restrict__ band_node, const T *__restrict__ band_w, int nbands,
                int n0, int n1, int BC, int nb_planes, int plane0, cplx_t<T> *__restrict__ G,
                cplx_t<T> *__restrict__ part)
{
    using C = cplx_t<T>;
    constexpr int FS = gather_fs_stride<P>();
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int next_tile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int R = 32 / BC, W = R + BC, nblk = n1 / BC;
    T *ws = (T *)(smraw + warp * gather_stage_bytes<T, P>(W));  // [32][W] weights
    C *fs = (C *)(ws + 32 * W);                                 // [32][FS] node values
    const int pb = blockIdx.y * P, np = min(P, nb_planes - pb);
    const int t0 = blockIdx.x * kGatherUnitsPerCta;
    const int t1 = min(nunits, t0 + kGatherUnitsPerCta);
    if (threadIdx.x == 0) next_tile = t0 + kGatherWarps;
    __syncthreads();
    const int rr = lane / BC, cc = lane - rr * BC;
    const int wv16 = W * (int)sizeof(T) / 16;  // 16-byte vectors of an entry's weights
    int it = t0 + warp;
    while (it < t1) {
        const int4 un = units[it];  // tile, first entry, end, partial slot (0: G)
        const int tile = un.x, beg = un.y, end = un.z;
        T ar[P], ai[P];
        Kahan2 ks[P];  // FP32: compensated totals of the chunk sums (re, im)
#pragma unroll
        for (int p = 0; p < P; p++) {
            ar[p] = ai[p] = T(0);
            ks[p].init();
        }
        for (int base = beg; base < end; base += 32) {
            const int n = min(32, end - base);
            if (lane < n) {
                const int e = base + lane;
                const int j = band_node[e];
                const float4 *src = reinterpret_cast<const float4 *>(band_w + (size_t)e * W);
                float4 *dst = reinterpret_cast<float4 *>(ws + lane * W);
                for (int q = 0; q < wv16; q++) dst[q] = src[q];
                const T wv = WEIGHTED ? sa.w[j] : T(1);
#pragma unroll
                for (int p = 0; p < P; p++) {
                    C fv = mkc<T>(0, 0);
                    if (p < np) {
                        fv = sa.f[(size_t)(plane0 + pb + p) * sa.f_stride + j];
                        if (WEIGHTED) fv = mkc<T>(wv * fv.x, wv * fv.y);
                    }
                    fs[lane * FS + p] = fv;
                }
            }
            __syncwarp();
            if constexpr (sizeof(T) == 4) {
                float2 bs[P];  // the chunk's sums (re, im) of each plane
#pragma unroll
                for (int p = 0; p < P; p++) bs[p] = make_float2(0.f, 0.f);
#pragma unroll 2
                for (int k = 0; k < n; k++) {
                    const float q = ws[k * W + rr] * ws[k * W + R + cc];
                    const float2 qq = make_float2(q, q);
                    if constexpr (P % 2 == 0) {
#pragma unroll
                        for (int p = 0; p < P; p += 2) {
                            const float4 f2 = *reinterpret_cast<const float4 *>(fs + k * FS + p);
                            bs[p] = __ffma2_rn(qq, make_float2(f2.x, f2.y), bs[p]);
                            bs[p + 1] = __ffma2_rn(qq, make_float2(f2.z, f2.w), bs[p + 1]);
                        }
                    } else {
#pragma unroll
                        for (int p = 0; p < P; p++) {
                            const C fv = fs[k * FS + p];
                            bs[p] = __ffma2_rn(qq, make_float2(fv.x, fv.y), bs[p]);
                        }
                    }
                }
#pragma unroll
                for (int p = 0; p < P; p++) ks[p].add(bs[p]);
            } else {
                // FP64: the point's weight once per entry, then one fused
                // multiply-add per plane and component (the FP64 pipe is
                // the bound on this GPU)
                for (int k = 0; k < n; k++) {
                    const T q = ws[k * W + rr] * ws[k * W + R + cc];
#pragma unroll
                    for (int p = 0; p < P; p++) {
                        const C fv = fs[k * FS + p];
                        ar[p] = fma(q, fv.x, ar[p]);
                        ai[p] = fma(q, fv.y, ai[p]);
                    }
                }
            }
            __syncwarp();  // the stage is refilled by the next chunk
        }
        const int b = tile / nbands, v = tile - b * nbands;
#pragma unroll
        for (int p = 0; p < P; p++) {
            if (p < np) {
                if (sizeof(T) == 4) {
                    const float2 v = ks[p].value();
                    ar[p] = (T)v.x;
                    ai[p] = (T)v.y;
                }
                const C val = mkc<T>(ar[p], ai[p]);
                if (un.w == 0)
                    G[(((size_t)(pb + p) * nblk + b) * n0 + (size_t)v * R) * BC + lane] = val;
                else
                    part[(((size_t)(un.w - 1) * nb_planes) + pb + p) * 32 + lane] = val;
            }
        }
        int nt = 0;
        if (lane == 0) nt = atomicAdd(&next_tile, 1);
        it = __shfl_sync(0xffffffffu, nt, 0);
    }
}

// The tiles whose lists were split into several ranges: their grid points
// get the later ranges' partial sums added in range order (FP32: Neumaier
// compensated).  fix[i] = {tile, first partial slot, number of slots}; one
// thread per (grid point of the tile, plane).
template <typename T>
__global__ void __launch_bounds__(256)
k_spread_fixup(const int4 *__restrict__ fix, int nbands, int n0, int n1, int BC,
               int nb_planes, const cplx_t<T> *__restrict__ part, cplx_t<T> *__restrict__ G)
{
    using C = cplx_t<T>;
    const int4 fx = fix[blockIdx.x];
    const int lane = threadIdx.x & 31, R = 32 / BC, nblk = n1 / BC;
    const int p = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (p >= nb_planes) return;
    const int b = fx.x / nbands, v = fx.x - b * nbands;
    C *g = G + (((size_t)p * nblk + b) * n0 + (size_t)v * R) * BC + lane;
    Comp<T> kr, ki;
    kr.init();
    ki.init();
    const C g0 = *g;
    kr.add(g0.x);
    ki.add(g0.y);
    for (int k = 0; k < fx.z; k++) {
        const C q = part[(((size_t)(fx.y - 1 + k) * nb_planes) + p) * 32 + lane];
        kr.add(q.x);
        ki.add(q.y);
    }
    *g = mkc<T>(kr.value(), ki.value());
}

// ================================================================ K1'/K5' row passes, four-step
// The row passes for n1 = R1 x R2 (256, 512, 1024): R2 threads per row,
// 128 / R2 rows per 128-thread CTA, each row's exchange buffer R1 x (R2 + 1)
// elements.  K1': deconvolve + zero-pad the N1 coefficients of the row
// straight into pass 1's registers (only the nonzero ones are loaded),
// forward FFT, all n1 outputs to H.  K5': the row of H' into registers,
// inverse FFT, the N1 kept outputs deconvolved into the coefficients plus
// the epilogue (|z|^2 partial per CTA, p = z).
template <int R1, int R2> __host__ __device__ constexpr int fs_row_stride() { return R1 * (R2 + 1); }

template <typename T, int MODE, int R1, int R2>
__global__ void __launch_bounds__(128)
k_rowfft_fs(const void *__restrict__ src, size_t src_stride, int N0, int N1,
            const T *__restrict__ c0, const T *__restrict__ c1, const cplx_t<T> *__restrict__ tw1,
            int plane0, cplx_t<T> *__restrict__ H, cplx_t<T> *__restrict__ f_init, size_t f_stride)
{
    using C = cplx_t<T>;
    constexpr int n1 = R1 * R2, RPC = 128 / R2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int line = threadIdx.x / R2, j = threadIdx.x - line * R2;
    C *S = (C *)smraw + line * fs_row_stride<R1, R2>();
    const int b = blockIdx.y, gb = plane0 + b, a = blockIdx.x * RPC + line;
    const bool live = a < N0;
    C x[R1];
    const T ca = live ? c0[a] : T(0);
#pragma unroll
    for (int m = 0; m < R1; m++) {
        const int l = j + R2 * m;
        const int k1 = l < n1 / 2 ? l : l - n1, c = k1 + N1 / 2;
        x[m] = mkc<T>(0, 0);
        if (live && c >= 0 && c < N1) {
            const size_t o = (size_t)gb * src_stride + (size_t)a * N1 + c;
            C sv;
            if (MODE == PM_COMPLEX) {
                sv = ((const C *)src)[o];
            } else {
                sv = mkc<T>(((const T *)src)[o], T(0));
                f_init[(size_t)gb * f_stride + (size_t)a * N1 + c] = sv;
            }
            const T sc = ca * c1[c];
            x[m] = mkc<T>(sv.x * sc, sv.y * sc);
        }
    }
    fs_dft<T, -1, R1>(x);
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) {
        C v = x[fs_out<R1>(k1)];
        if (k1) v = cmul<T>(v, tw1[j * k1]);
        S[k1 * (R2 + 1) + j] = v;
    }
    __syncthreads();
    if (!live) return;
    C *Hrow = H + ((size_t)b * N0 + a) * n1;
    for (int k1 = j; k1 < R1; k1 += R2) {
        C y[R2];
#pragma unroll
        for (int jj = 0; jj < R2; jj++) y[jj] = S[k1 * (R2 + 1) + jj];
        fs_dft<T, -1, R2>(y);
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) Hrow[k1 + R1 * k2] = y[fs_out<R2>(k2)];
    }
}

template <typename T, int MODE, int R1, int R2>
__global__ void __launch_bounds__(128)
k_rowifft_crop_fs(const cplx_t<T> *__restrict__ Hp, int N0, int N1, const T *__restrict__ c0,
                  const T *__restrict__ c1, const cplx_t<T> *__restrict__ tw1, int plane0,
                  CropArgs<T> ca)
{
    using C = cplx_t<T>;
    constexpr int n1 = R1 * R2, RPC = 128 / R2;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double sh[32];
    const int line = threadIdx.x / R2, j = threadIdx.x - line * R2;
    C *S = (C *)smraw + line * fs_row_stride<R1, R2>();
    const int b = blockIdx.y, gb = plane0 + b, a = blockIdx.x * RPC + line;
    const bool live = a < N0;
    const C *Hrow = Hp + ((size_t)b * N0 + (live ? a : 0)) * n1;
    C x[R1];
#pragma unroll
    for (int m = 0; m < R1; m++) x[m] = live ? Hrow[j + R2 * m] : mkc<T>(0, 0);
    fs_dft<T, +1, R1>(x);
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) {
        C v = x[fs_out<R1>(k1)];
        if (k1) {
            C w = tw1[j * k1];
            w.y = -w.y;
            v = cmul<T>(v, w);
        }
        S[k1 * (R2 + 1) + j] = v;
    }
    __syncthreads();
    T s = 0;
    if (live) {
        const T sa = c0[a];
        for (int k1 = j; k1 < R1; k1 += R2) {
            C y[R2];
#pragma unroll
            for (int jj = 0; jj < R2; jj++) y[jj] = S[k1 * (R2 + 1) + jj];
            fs_dft<T, +1, R2>(y);
#pragma unroll
            for (int k2 = 0; k2 < R2; k2++) {
                // output index l1 = k1 + R1 k2 is column c = l1 + N1/2 (mod n1)
                int c = k1 + R1 * k2 + N1 / 2;
                if (c >= n1) c -= n1;
                if (c < N1) {
                    const C g = y[fs_out<R2>(k2)];
                    const size_t o = (size_t)gb * ca.out_stride + (size_t)a * N1 + c;
                    if (MODE == CM_TRESID) {
                        // z = b - T f (b in out), p = z
                        const C bv = ca.out[o];
                        const C z = mkc<T>(bv.x - g.x, bv.y - g.y);
                        ca.out[o] = z;
                        ca.p_out[o] = z;
                        s += z.x * z.x + z.y * z.y;
                    } else if (MODE == CM_TPDOT) {
                        // q = T p, Re(p^H q)
                        const C pv = ca.pin[o];
                        ca.out[o] = g;
                        s += pv.x * g.x + pv.y * g.y;
                    } else {
                        const T sc = sa * c1[c];
                        const C z = mkc<T>(g.x * sc, g.y * sc);
                        ca.out[o] = z;
                        if (MODE == CM_INIT) ca.p_out[o] = z;
                        s += z.x * z.x + z.y * z.y;
                    }
                }
            }
        }
    }
    if (MODE != CM_PLAIN) {
        const double d = block_sum_t<T>(s, sh);
        if (threadIdx.x == 0) ca.part[(size_t)gb * ca.part_stride + blockIdx.x] = d;
    }
}

// ================================================================ K4b' column IFFT, four-step
// The column IFFT for n0 = R1 x R2 (256, 512, 1024): one CTA per (column
// block of 4 columns, plane), R2 threads per column.  Pass 1 reads the grid
// straight from G into registers (a warp reads 8 rows x 4 columns, 256
// contiguous bytes, per step), the exchange goes through shared memory
// (column stride padded so neither pass meets a bank twice), pass 2 writes
// the N0 kept rows to H'.

// shared memory of k_colfft_interp_fs: four columns of n0 + 8 plus the exchange
template <typename T> static size_t smem_colfs_of(int R1, int R2)
{
    const int cs = R1 == 32 && R2 == 32   ? fs_col_stride<32, 32>()
                   : R1 == 32 && R2 == 16 ? fs_col_stride<32, 16>()
                                          : fs_col_stride<16, 16>();
    return sizeof(cplx_t<T>) * 4 * ((size_t)R1 * R2 + 8 + cs);
}

template <typename T, int R1, int R2>
__global__ void __launch_bounds__(4 * R2)
k_colifft_fs(const cplx_t<T> *__restrict__ G, int N0, int n1, const cplx_t<T> *__restrict__ tw0,
             cplx_t<T> *__restrict__ Hp)
{
    using C = cplx_t<T>;
    constexpr int n0 = R1 * R2, BC = 4, CS = fs_col_stride<R1, R2>();
    extern __shared__ __align__(16) unsigned char smraw[];
    C *S = (C *)smraw;  // [column][k1][j], column stride CS, row stride R2 + 1
    const int cb = blockIdx.x, b = blockIdx.y, nblk = n1 / BC;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = lane & 3, j = warp * 8 + (lane >> 2);
    const C *Gb = G + ((size_t)b * nblk + cb) * n0 * BC;
    {
        C a[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) a[m] = Gb[(size_t)(j + R2 * m) * BC + c];
        fs_dft<T, +1, R1>(a);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            C v = a[fs_out<R1>(k1)];
            if (k1) {
                C w = tw0[j * k1];
                w.y = -w.y;  // inverse: e^{+2 pi i j k1 / n0}
                v = cmul<T>(v, w);
            }
            S[c * CS + k1 * (R2 + 1) + j] = v;
        }
    }
    __syncthreads();
    C *Hb = Hp + (size_t)b * N0 * n1 + (size_t)cb * BC + c;
    for (int k1 = j; k1 < R1; k1 += R2) {
        C y[R2];
#pragma unroll
        for (int jj = 0; jj < R2; jj++) y[jj] = S[c * CS + k1 * (R2 + 1) + jj];
        fs_dft<T, +1, R2>(y);
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) {
            const int a = (k1 + R1 * k2 + N0 / 2) & (n0 - 1);
            if (a < N0) Hb[(size_t)a * n1] = y[fs_out<R2>(k2)];
        }
    }
}

// ================================================================ Toeplitz column pass
// CGNR's normal operator T = A^H W A is a convolution on the N0 x N1
// coefficients: (T p)[k] = sum_k' K[k - k'] p[k'], K[m] = sum_j w_j
// e^{2 pi i m x_j}, |m| < N.  Embedded in the n0 x n1 circulant (n >= 2N - 1,
// so no wrap reaches a kept output) it is a pointwise product of DFTs: row
// FFT of the zero-padded rows (K1' with unit factors), then per column the
// n0-point FFT, the product with khat (the kernel's DFT / (n0 n1)) and the
// inverse FFT, keeping the N0 rows (this kernel), then the inverse row FFT
// with the crop (K5' with unit factors).  One CTA per (4-column block,
// plane), R2 threads per column: pass 1 as in k_colfft_interp_fs; pass 2
// leaves thread k1 with Y[k1 + R1 k2] for all k2, which is the first
// (R2-point, over k2) step of the inverse four-step FFT: its outputs t2 are
// twiddled by e^{+2 pi i k1 t2 / n0} and exchanged, and thread t2 finishes
// with the R1-point DFT over k1 (output row t2 + R2 t1).  The exchange buffer
// is reused for the inverse (one barrier between the last read and the first
// write).  In place: the CTA reads and writes the same N0 x 4 values of H.
// Three CTAs per SM (168 registers; capping the 768-point form at 128
// registers for a fourth CTA made the passes slower, 14.4 -> 16.5 ms per
// cfg2 iteration).
template <typename T, int R1, int R2>
__global__ void __launch_bounds__(4 * R2, 3)
k_col_toeplitz(cplx_t<T> *__restrict__ H, int N0, int n1, const cplx_t<T> *__restrict__ tw0,
               const cplx_t<T> *__restrict__ khat)
{
    using C = cplx_t<T>;
    constexpr int n0 = R1 * R2, BC = 4, CS = fs_col_stride<R1, R2>(), KI = (R1 + R2 - 1) / R2;
    static_assert(R2 * (R1 + 1) <= CS, "inverse exchange exceeds the column stride");
    extern __shared__ __align__(16) unsigned char smraw[];
    C *S = (C *)smraw;
    const int cb = blockIdx.x, b = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = lane & 3, j = warp * 8 + (lane >> 2);
    C *Hb = H + (size_t)b * N0 * n1 + (size_t)cb * BC + c;
    {
        C x[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
            const int l0 = j + R2 * m;
            const int a = (l0 < n0 / 2 ? l0 : l0 - n0) + N0 / 2;
            x[m] = (a >= 0 && a < N0) ? Hb[(size_t)a * n1] : mkc<T>(0, 0);
        }
        fs_dft<T, -1, R1>(x);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            C v = x[fs_out<R1>(k1)];
            if (k1) v = cmul<T>(v, tw0[j * k1]);
            S[c * CS + k1 * (R2 + 1) + j] = v;
        }
    }
    __syncthreads();
    C y[KI][R2];
#pragma unroll
    for (int i = 0; i < KI; i++)
        if (j + R2 * i < R1)
#pragma unroll
            for (int jj = 0; jj < R2; jj++) y[i][jj] = S[c * CS + (j + R2 * i) * (R2 + 1) + jj];
    __syncthreads();  // S is reused for the inverse exchange
#pragma unroll
    for (int i = 0; i < KI; i++) {
        const int k1 = j + R2 * i;
        if (k1 >= R1) break;
        fs_dft<T, -1, R2>(y[i]);
        C z[R2];
        const C *kp = khat + (((size_t)cb * R2) * R1 + k1) * BC + c;
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++)
            z[k2] = cmul<T>(y[i][fs_out<R2>(k2)], kp[(size_t)k2 * R1 * BC]);
        fs_dft<T, +1, R2>(z);
#pragma unroll
        for (int t2 = 0; t2 < R2; t2++) {
            C v = z[fs_out<R2>(t2)];
            if (k1 * t2) {
                C w = tw0[k1 * t2];
                w.y = -w.y;  // inverse: e^{+2 pi i k1 t2 / n0}
                v = cmul<T>(v, w);
            }
            S[c * CS + t2 * (R1 + 1) + k1] = v;
        }
    }
    __syncthreads();
    {
        const int t2 = j;
        C w[R1];
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) w[k1] = S[c * CS + t2 * (R1 + 1) + k1];
        fs_dft<T, +1, R1>(w);
#pragma unroll
        for (int t1 = 0; t1 < R1; t1++) {
            int a = t2 + R2 * t1 + N0 / 2;
            if (a >= n0) a -= n0;
            if (a < N0) Hb[(size_t)a * n1] = w[fs_out<R1>(t1)];
        }
    }
}

// The operator's kernel in FP64 from the polar set's factored form: node
// (a, i) = r_i (sg_a, cg_a) and weight w_i, so K[m] = sum_a G(m0 sg_a + m1
// cg_a) with G(s) = sum_i w_i e^{2 pi i r_i s}.  G is tabulated at s_k =
// (k - K0) delta (one thread per k, the radii summed in order) and read back
// by 8-point Lagrange interpolation: G has at most half a turn per unit of s
// (|r| <= 1/2), so delta = 1/32 leaves ~1e-11 relative error.
__global__ void k_toep_gtable(const double *__restrict__ r, const double *__restrict__ w, int np,
                              double delta, int K0, int Ns, double2 *__restrict__ G)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Ns) return;
    const double sv = (k - K0) * delta;
    double re = 0, im = 0;
    for (int i = 0; i < np; i++) {
        double sn, cs;
        sincospi(2.0 * r[i] * sv, &sn, &cs);
        const double wi = w ? w[i] : 1.0;
        re = fma(wi, cs, re);
        im = fma(wi, sn, im);
    }
    G[k] = make_double2(re, im);
}

// circ[l0][l1] = K[m] for the signed indices m = (l0, l1) (mod nt) with
// |m0| < N0, |m1| < N1, else 0; the lines summed in order.  The weights are
// real, so K[-m] = conj(K[m]): a thread takes the m of rows l0 <= nt/2 (for
// row 0 and row nt/2 the columns l1 <= nt/2) and also writes -m; every entry
// is written once.
__global__ void k_toep_circ(const double2 *__restrict__ G, double delta, int K0,
                            const double *__restrict__ sg, const double *__restrict__ cg, int A,
                            int N0, int N1, int nt, double2 *__restrict__ circ)
{
    const int h = nt / 2;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)(h + 1) * nt) return;
    const int l0 = (int)(i / nt), l1 = (int)(i - (size_t)l0 * nt);
    if ((l0 == 0 || l0 == h) && l1 > h) return;  // the mirror of a column l1 < h
    const int m0 = l0 < h ? l0 : l0 - nt, m1 = l1 < h ? l1 : l1 - nt;
    double re = 0, im = 0;
    if (m0 > -N0 && m0 < N0 && m1 > -N1 && m1 < N1) {
        // reciprocals of the Lagrange weights' denominators for the nodes
        // -3..4: 1 / prod_{l != j} (j - l)
        constexpr double rden[8] = {-1.0 / 5040, 1.0 / 720, -1.0 / 240, 1.0 / 144,
                                    -1.0 / 144,  1.0 / 240, -1.0 / 720, 1.0 / 5040};
        const double inv = 1.0 / delta;
        for (int a = 0; a < A; a++) {
            const double u = fma((double)m0, sg[a], (double)m1 * cg[a]) * inv + K0;
            const double fu = floor(u);
            const double t = u - fu;  // in [0, 1): nodes at t - (j - 3)
            const int k0 = (int)fu - 3;
            double d[8], pre[8], suf[8];
#pragma unroll
            for (int j = 0; j < 8; j++) d[j] = t - (j - 3);
            pre[0] = 1.0;
#pragma unroll
            for (int j = 1; j < 8; j++) pre[j] = pre[j - 1] * d[j - 1];
            suf[7] = 1.0;
#pragma unroll
            for (int j = 6; j >= 0; j--) suf[j] = suf[j + 1] * d[j + 1];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const double wj = pre[j] * suf[j] * rden[j];
                const double2 gv = G[k0 + j];
                re = fma(wj, gv.x, re);
                im = fma(wj, gv.y, im);
            }
        }
    }
    circ[i] = make_double2(re, im);
    const int r0 = l0 ? nt - l0 : 0, r1 = l1 ? nt - l1 : 0;  // -m (mod nt)
    if (r0 != l0 || r1 != l1) circ[(size_t)r0 * nt + r1] = make_double2(re, -im);
}

// The circulant's DFT (row-major nt x nt, FP64) divided by nt^2, in the
// order k_col_toeplitz<R1, R2> reads it: [block of 4 columns][k2][k1][column],
// frequency row l0 = k1 + R1 k2.
template <typename T>
__global__ void k_toep_layout(const double2 *__restrict__ F, int n0, int n1, int R1, int R2,
                              cplx_t<T> *__restrict__ khat)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n0 * n1) return;
    const int l0 = (int)(i / n1), l1 = (int)(i - (size_t)l0 * n1);
    const int k1 = l0 % R1, k2 = l0 / R1, cb = l1 >> 2, c = l1 & 3;
    const double sc = 1.0 / ((double)n0 * (double)n1);
    const double2 v = F[i];
    khat[(((size_t)cb * R2 + k2) * R1 + k1) * 4 + c] = mkc<T>((T)(v.x * sc), (T)(v.y * sc));
}

// ================================================================ K4b column IFFT
// One CTA per (column block, plane): the block's n0 x BC grid values (one
// contiguous run of G) into shared memory column by column, BC inverse
// n0-point FFTs, the N0 kept rows (a - N0/2 mod n0) written to H'.
template <typename T>
__global__ void __launch_bounds__(256)
k_colifft(const cplx_t<T> *__restrict__ G, int N0, int n0, int logn0, int n1, int BC,
          const cplx_t<T> *__restrict__ tw0, cplx_t<T> *__restrict__ Hp)
{
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *A = (C *)smraw, *B = A + fft_buf((size_t)BC * n0);
    const int cb = blockIdx.x, b = blockIdx.y, nblk = n1 / BC;
    const C *Gb = G + ((size_t)b * nblk + cb) * n0 * BC;
    // row l0's BC values are contiguous: thread l0 moves them to the BC
    // columns (consecutive threads, consecutive rows: no bank conflicts);
    // four (FP32) or two (FP64) rows per thread in flight
    {
        constexpr int U = sizeof(T) == 4 ? 4 : 2;
        for (int base = threadIdx.x; base < n0; base += U * blockDim.x) {
            C v[U][4];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int l0 = base + u * blockDim.x;
                if (l0 < n0)
                    for (int c = 0; c < BC && c < 4; c++) v[u][c] = Gb[(size_t)l0 * BC + c];
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int l0 = base + u * blockDim.x;
                if (l0 < n0)
                    for (int c = 0; c < BC && c < 4; c++) A[(size_t)c * n0 + l0] = v[u][c];
            }
        }
        for (int c = 4; c < BC; c++)  // blocks wider than 4 columns
            for (int l0 = threadIdx.x; l0 < n0; l0 += blockDim.x)
                A[(size_t)c * n0 + l0] = Gb[(size_t)l0 * BC + c];
    }
    __syncthreads();
    const C *R = block_fft<T, +1>(A, B, n0, logn0, BC, tw0);
    C *Hb = Hp + (size_t)b * N0 * n1 + (size_t)cb * BC;
    for (int idx = threadIdx.x; idx < N0 * BC; idx += blockDim.x) {
        const int a = idx / BC, cl = idx - a * BC;
        const int l0 = (a - N0 / 2) & (n0 - 1);
        Hb[(size_t)a * n1 + cl] = R[(size_t)cl * n0 + l0];
    }
}

// ================================================================ K5 row IFFT + crop
template <typename T, int MODE>
__global__ void __launch_bounds__(256)
k_rowifft_crop(const cplx_t<T> *__restrict__ Hp, int N0, int N1, int n1, int logn1, int kRows,
               const T *__restrict__ c0, const T *__restrict__ c1,
               const cplx_t<T> *__restrict__ tw1, int plane0, CropArgs<T> ca)
{
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double sh[32];
    C *A = (C *)smraw, *B = A + fft_buf((size_t)kRows * n1);
    int b = blockIdx.y, gb = plane0 + b, a0 = blockIdx.x * kRows;
    int nr = min(kRows, N0 - a0);
    const C *Hb = Hp + ((size_t)b * N0 + a0) * n1;
    {
        // the nr contiguous rows as 16-byte vectors, eight per thread in
        // flight before the shared-memory stores
        using V = float4;
        const int nv = nr * n1 * (int)sizeof(C) / 16;
        const V *src = reinterpret_cast<const V *>(Hb);
        V *dst = reinterpret_cast<V *>(A);
        constexpr int U = 8;
        for (int base = threadIdx.x; base < nv; base += U * blockDim.x) {
            V v[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int i = base + u * blockDim.x;
                if (i < nv) v[u] = src[i];
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int i = base + u * blockDim.x;
                if (i < nv) dst[i] = v[u];
            }
        }
    }
    __syncthreads();
    C *R = block_fft<T, +1>(A, B, n1, logn1, nr, tw1);
    T s = 0;
    for (int idx = threadIdx.x; idx < nr * N1; idx += blockDim.x) {
        int r = idx / N1, c = idx - r * N1;
        int a = a0 + r;
        int l1 = (c - N1 / 2) & (n1 - 1);
        C g = R[r * n1 + l1];
        T sc = c0[a] * c1[c];
        C z = mkc<T>(g.x * sc, g.y * sc);
        size_t o = (size_t)gb * ca.out_stride + (size_t)a * N1 + c;
        ca.out[o] = z;
        if (MODE == CM_INIT) ca.p_out[o] = z;
        s += z.x * z.x + z.y * z.y;
    }
    if (MODE != CM_PLAIN) {
        double d = block_sum_t<T>(s, sh);
        if (threadIdx.x == 0) ca.part[(size_t)gb * ca.part_stride + blockIdx.x] = d;
    }
}

// ================================================================ host side
static int ilog2(int n)
{
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

template <typename T> int NfftDev<T>::init_fused(const NfftTables &t, cudaStream_t st)
{
    // column-block width: two BC x n0 complex buffers within 128 KB, at most
    // 4 columns (measured: two 4-column CTAs per SM beat one 8-column CTA)
    int bc = (int)((128 << 10) / (2 * sizeof(C) * (size_t)t.n0));
    if (bc > 4) bc = 4;
    // the FP32 four-step column pass takes 8-column blocks (fewer entries)
    if (sizeof(T) == 4 && (t.n0 == 1024 || t.n0 == 512 || t.n0 == 256) && t.n1 >= 64) bc = 8;
    if (bc > t.n1) bc = t.n1;
    // the autotuner's cap, else NUDIM_TUNE_BC (a tuning knob: narrower blocks
    // fit more CTAs per SM at the cost of more (node, block) entries)
    {
        int v = tune_bc;
        if (!v)
            if (const char *e = getenv("NUDIM_TUNE_BC")) v = atoi(e);
        if (v >= 1 && v < bc) bc = v;
    }
    int p = 1;
    while (p * 2 <= bc) p *= 2;
    bc = p;
    if (bc < 1) return NUDIM_EINVAL;
    // a window must not wrap onto its own block: narrow grids use one block
    if (t.n1 < kW - 1 + bc && t.n1 <= 32 && 2 * sizeof(C) * (size_t)t.n1 * t.n0 <= (128u << 10))
        bc = t.n1;
    // adjoint: blocks of 4 columns (tiles of 8 x 4 grid points; the tile's
    // 12 weights move as 16-byte vectors)
    if (t.n1 < 4 || t.n0 < 8) return NUDIM_EINVAL;
    const int bca = 4;
    FusedLists<T> L;
    if (build_fused_lists(t, bc, bca, sizeof(T) == 4, &L, !trafo_only) != 0) {
        set_error("fused NFFT list construction failed");
        return NUDIM_EINVAL;
    }
    BC = L.BC;
    nblk = L.nblk;
    smax = L.smax;
    BCa = L.BCa;
    nblka = L.nblka;
    nbands = L.nbands;
    ntiles = nblka * nbands;
    // spreading work units: every tile's list in ranges of at most
    // kGatherMaxEntries entries (split evenly), longest range first; the
    // tiles of more than one range, with their partial slots, for the fix-up
    std::vector<int4> hu, hf;
    nextra = 0;
    for (int i = 0; i < (trafo_only ? 0 : ntiles); i++) {
        const int t = L.band_ord[i], b0 = L.band_off[t], len = L.band_off[t + 1] - b0;
        const int nr = std::max(1, ceil_div(len, kGatherMaxEntries));
        for (int r = 0; r < nr; r++)
            hu.push_back(make_int4(t, b0 + (int)((long)len * r / nr),
                                   b0 + (int)((long)len * (r + 1) / nr), r ? nextra + r : 0));
        if (nr > 1) {
            hf.push_back(make_int4(t, nextra + 1, nr - 1, 0));
            nextra += nr - 1;
        }
    }
    std::stable_sort(hu.begin(), hu.end(),
                     [](const int4 &a, const int4 &b) { return a.z - a.y > b.z - b.y; });
    nunits = (int)hu.size();
    nfix = (int)hf.size();
    // rows per CTA in the row passes: two (padded) rows x n1 complex buffers within 112 KB
    rows = 4;
    while (rows > 1 && 2 * sizeof(C) * fft_buf((size_t)rows * t.n1) > ((size_t)112 << 10)) rows--;
    smem_col = 2 * sizeof(C) * fft_buf((size_t)BC * n0);
    smem_row = 2 * sizeof(C) * fft_buf((size_t)rows * n1);
    // row passes as four-step FFTs where n1 = R1 x R2 is 256, 512 or 1024:
    // 128 / R2 rows per CTA (the CTA count also sets the crop pass's number
    // of partial sums per plane)
    row_fs = n1 == 1024 || n1 == 512 || n1 == 256;
    if (row_fs) {
        const int r1 = n1 == 256 ? 16 : 32, r2 = n1 / r1;
        rows = 128 / r2;
        smem_row = sizeof(C) * (size_t)rows * r1 * (r2 + 1);
    }
    // adjoint: planes per gather pass 8 (default), 4, 2 or 1 -- the
    // autotuner's cap, else NUDIM_TUNE_PLANES
    Pa = 8;
    {
        int v = tune_planes;
        if (!v)
            if (const char *e = getenv("NUDIM_TUNE_PLANES")) v = atoi(e);
        if (v >= 1 && v < 8) Pa = v >= 4 ? 4 : v >= 2 ? 2 : 1;
    }
    const int Wa = 32 / BCa + BCa;
    smem_spread = kGatherWarps * (Pa == 8   ? gather_stage_bytes<T, 8>(Wa)
                                  : Pa == 4 ? gather_stage_bytes<T, 4>(Wa)
                                  : Pa == 2 ? gather_stage_bytes<T, 2>(Wa)
                                            : gather_stage_bytes<T, 1>(Wa));
    smem_colifft = 2 * sizeof(C) * fft_buf((size_t)BCa * n0);
    // The limit is a property of the kernel, shared by every plan in the
    // process: set it to the largest size any plan uses (never lower it).
    const int lim_col = 144 << 10, lim_row = 112 << 10, lim_spread = 96 << 10,
              lim_colifft = 144 << 10;
    if (rows < 1 || smem_col > (size_t)lim_col || smem_row > (size_t)lim_row ||
        smem_spread > (size_t)lim_spread || smem_colifft > (size_t)lim_colifft) {
        set_error("fused NFFT: shared memory plan exceeds the kernel limits");
        return NUDIM_EINVAL;
    }
    std::vector<double> w0, w1;
    fft_twiddles(n0, &w0);
    fft_twiddles(n1, &w1);
    std::vector<T> t0(w0.begin(), w0.end()), t1(w1.begin(), w1.end());
    auto up = [&](void **dst, const void *srcp, size_t nb) -> int {
        bytes += nb;
        return upload_async(dst, srcp, nb, st);
    };
    NUDIM_TRY(up((void **)&tw0, t0.data(), sizeof(T) * t0.size()));
    NUDIM_TRY(up((void **)&tw1, t1.data(), sizeof(T) * t1.size()));
    NUDIM_TRY(up((void **)&blk_off, L.blk_off.data(), sizeof(int) * L.blk_off.size()));
    NUDIM_TRY(up((void **)&ent, L.ent.data(), sizeof(int) * L.ent.size()));
    NUDIM_TRY(up((void **)&nslots, L.nslots.data(), L.nslots.size()));
    nE = (int)L.ent.size();
    if (L.ent_rb.empty()) L.ent_rb.assign(1, 0);
    if (L.ent_cc.empty()) L.ent_cc.assign(1, 0);
    NUDIM_TRY(up((void **)&e_rb, L.ent_rb.data(), sizeof(int) * L.ent_rb.size()));
    NUDIM_TRY(up((void **)&e_cc, L.ent_cc.data(), sizeof(int) * L.ent_cc.size()));
    NUDIM_TRY(up((void **)&e_qa, L.ent_qa.data(), sizeof(T) * L.ent_qa.size()));
    NUDIM_TRY(up((void **)&e_q1, L.ent_q1.data(), sizeof(T) * L.ent_q1.size()));
    NUDIM_TRY(up((void **)&band_off, L.band_off.data(), sizeof(int) * L.band_off.size()));
    NUDIM_TRY(up((void **)&band_node, L.band_node.data(),
                 sizeof(int) * std::max<size_t>(1, L.band_node.size())));
    NUDIM_TRY(up((void **)&units, hu.data(), sizeof(int4) * hu.size()));
    if (!hf.empty()) NUDIM_TRY(up((void **)&fixups, hf.data(), sizeof(int4) * hf.size()));
    NUDIM_TRY(up((void **)&band_w, L.band_w.data(), sizeof(T) * L.band_w.size()));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    lim_col));
    {
        const void *gk[] = {(const void *)k_spread_gather<T, true, 8>,
                            (const void *)k_spread_gather<T, false, 8>,
                            (const void *)k_spread_gather<T, true, 4>,
                            (const void *)k_spread_gather<T, false, 4>,
                            (const void *)k_spread_gather<T, true, 2>,
                            (const void *)k_spread_gather<T, false, 2>,
                            (const void *)k_spread_gather<T, true, 1>,
                            (const void *)k_spread_gather<T, false, 1>};
        for (const void *k : gk)
            NUDIM_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            lim_spread));
    }
    NUDIM_CUDA(cudaFuncSetAttribute(k_colifft<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    lim_colifft));
    {
        // the four-step row passes' exchange buffers (FP64 1024 points: 68 KB)
        const int lr1 = (int)(sizeof(C) * 4 * fs_row_stride<32, 32>());
        const int lr2 = (int)(sizeof(C) * 8 * fs_row_stride<32, 16>());
        const int lr3 = (int)(sizeof(C) * 8 * fs_row_stride<16, 16>());
#define NUDIM_ROWFS_ATTR(R1, R2, L)                                                              \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowfft_fs<T, PM_COMPLEX, R1, R2>,                          \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L));           \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowfft_fs<T, PM_REAL_INIT, R1, R2>,                        \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L));           \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_PLAIN, R1, R2>,                      \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L));           \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_DOT, R1, R2>,                        \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L));           \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_INIT, R1, R2>,                       \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L));           \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_TRESID, R1, R2>,                     \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L));           \
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_TPDOT, R1, R2>,                      \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, L))
        NUDIM_ROWFS_ATTR(32, 32, lr1);
        NUDIM_ROWFS_ATTR(32, 16, lr2);
        NUDIM_ROWFS_ATTR(16, 16, lr3);
#undef NUDIM_ROWFS_ATTR
    }
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs8<32, 32>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs8<32, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs8<16, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs2<32, 32>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs2<32, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs2<16, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs<T, 32, 32>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs<T, 32, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colfft_interp_fs<T, 16, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_col));
    // the four-step column IFFTs' exchange buffers (FP64 1024 points: 68 KB)
    NUDIM_CUDA(cudaFuncSetAttribute(k_col_toeplitz<T, 32, 32>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<32, 32>())));
    NUDIM_CUDA(cudaFuncSetAttribute(k_col_toeplitz<T, 32, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<32, 16>())));
    NUDIM_CUDA(cudaFuncSetAttribute(k_col_toeplitz<T, 16, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<16, 16>())));
    NUDIM_CUDA(cudaFuncSetAttribute(k_col_toeplitz<T, 24, 32>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<24, 32>())));
    {
        // the 768-point circulant's row passes (24 x 32)
        const int lt = (int)(sizeof(C) * 4 * fs_row_stride<24, 32>());
        NUDIM_CUDA(cudaFuncSetAttribute(k_rowfft_fs<T, PM_COMPLEX, 24, 32>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, lt));
        NUDIM_CUDA(cudaFuncSetAttribute(k_rowfft_fs<T, PM_REAL_INIT, 24, 32>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, lt));
        NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_PLAIN, 24, 32>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, lt));
        NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_TRESID, 24, 32>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, lt));
        NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop_fs<T, CM_TPDOT, 24, 32>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, lt));
    }
    NUDIM_CUDA(cudaFuncSetAttribute(k_colifft_fs<T, 32, 32>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<32, 32>())));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colifft_fs<T, 32, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<32, 16>())));
    NUDIM_CUDA(cudaFuncSetAttribute(k_colifft_fs<T, 16, 16>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(C) * 4 * fs_col_stride<16, 16>())));
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowfft<T, PM_COMPLEX>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_row));
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowfft<T, PM_REAL_INIT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_row));
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop<T, CM_PLAIN>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_row));
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop<T, CM_DOT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_row));
    NUDIM_CUDA(cudaFuncSetAttribute(k_rowifft_crop<T, CM_INIT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, lim_row));
    fused = true;
    return NUDIM_OK;
}

template <typename T> void NfftDev<T>::release_fused()
{
    void *ptrs[] = {tw0,    tw1,  blk_off, ent,  nslots, band_off, band_node,
                    units,  band_w, e_rb, e_cc, e_qa, e_q1, fixups, khat, ones};
    if (twT && twT != tw0) cudaFreeAsync(twT, ast);
    twT = nullptr;
    nT = 0;
    khat = nullptr;
    ones = nullptr;
    toeplitz = false;
    for (void *q : ptrs)
        if (q) cudaFreeAsync(q, ast);
    tw0 = tw1 = nullptr;
    blk_off = ent = band_off = band_node = e_rb = e_cc = nullptr;
    units = fixups = nullptr;
    band_w = e_qa = e_q1 = nullptr;
    nslots = nullptr;
    fused = false;
}

// Planes per fused pass: the pass's scratch per plane (complex elements:
// trafo N0*n1 row spectra + smax*M partials, adjoint N0*n1 + n0*n1 grid)
// within the context's budget.
template <typename T> int NfftDev<T>::fused_chunk(int nplanes, size_t per_plane) const
{
    size_t per = sizeof(C) * per_plane;
    size_t budget = ctx->fused_budget ? ctx->fused_budget : ((size_t)3072 << 20);
    long c = (long)(budget / per);
    if (c < 1) c = 1;
    if (c > nplanes) c = nplanes;
    return (int)c;
}

// Algorithmic bytes per launch (profiler), c = complex size:
//   row pass  nb*c*(N0*N1 + N0*n1)     coefficients in, row spectra out
//   col pass  nb*c*(N0*n1 + smax*M)    row spectra in, partials out (+ tables)
//   combine   nb*c*(smax*M + M)        partials in, node values out
template <typename T>
int NfftDev<T>::trafo_fused(int nplanes, const PadArgs<T> &pa, const InterpArgs<T> &ia,
                            cudaStream_t st)
{
    int chunk = fused_chunk(nplanes, (size_t)N0 * n1 + (size_t)smax * M);
    void *wsv;
    size_t nH = (size_t)N0 * n1 * chunk, nP = (size_t)smax * M * chunk;
    NUDIM_TRY(workspace(sizeof(C) * (nH + nP), &wsv));
    C *H = (C *)wsv, *P = H + nH;
    int logn0 = ilog2(n0), logn1 = ilog2(n1);
    const double c = sizeof(C), tab = (double)M * (8 + 2 * kW * sizeof(T));
    for (int p0 = 0; p0 < nplanes; p0 += chunk) {
        int nb = std::min(chunk, nplanes - p0);
        {
            ProfScope ps(ctx, PK_PAD, st, nb * c * ((double)N0 * N1 + (double)N0 * n1));
            dim3 g(ceil_div(N0, rows), nb);
#define NUDIM_ROWFS(MD, R1, R2)                                                                  \
    k_rowfft_fs<T, MD, R1, R2><<<g, 128, smem_row, st>>>(pa.src, pa.src_stride, N0, N1, c0, c1, \
                                                          tw1, p0, H, pa.f_init, pa.f_stride)
            if (row_fs) {
                if (pa.mode == PM_COMPLEX) {
                    if (n1 == 1024) NUDIM_ROWFS(PM_COMPLEX, 32, 32);
                    else if (n1 == 512) NUDIM_ROWFS(PM_COMPLEX, 32, 16);
                    else NUDIM_ROWFS(PM_COMPLEX, 16, 16);
                } else {
                    if (n1 == 1024) NUDIM_ROWFS(PM_REAL_INIT, 32, 32);
                    else if (n1 == 512) NUDIM_ROWFS(PM_REAL_INIT, 32, 16);
                    else NUDIM_ROWFS(PM_REAL_INIT, 16, 16);
                }
            } else if (pa.mode == PM_COMPLEX)
#undef NUDIM_ROWFS
                k_rowfft<T, PM_COMPLEX><<<g, 256, smem_row, st>>>(pa.src, pa.src_stride, N0, N1,
                                                                   n1, logn1, rows, c0, c1, tw1,
                                                                   p0, H, nullptr, 0);
            else
                k_rowfft<T, PM_REAL_INIT><<<g, 256, smem_row, st>>>(pa.src, pa.src_stride, N0,
                                                                     N1, n1, logn1, rows, c0, c1,
                                                                     tw1, p0, H, pa.f_init,
                                                                     pa.f_stride);
            NUDIM_LAUNCH_CHECK();
        }
        {
            ProfScope ps(ctx, PK_INTERP, st,
                         tab + nb * c * ((double)N0 * n1 + (double)smax * M));
            // one radix-16 butterfly per thread: 64 threads per column
            const int thr = std::min(32 * col_warps<T>(), std::max(64, 64 * BC));
#define NUDIM_COLFS(R1, R2)                                                                      \
    k_colfft_interp_fs<T, R1, R2><<<dim3(nblk, nb), thr, smem_colfs_of<T>(R1, R2), st>>>(             \
        H, N0, n1, tw0, blk_off, ent, e_rb, e_cc, e_qa, e_q1, nE, M, smax, P)
#define NUDIM_COLFS2(R1, R2)                                                                     \
    k_colfft_interp_fs2<R1, R2><<<dim3(nblk, ceil_div(nb, 2)), 256,                             \
                                  sizeof(float2) * 2 * 4 * fs2_gs<R1, R2>(), st>>>(             \
        (const float2 *)H, N0, n1, nb, (const float2 *)tw0, blk_off, ent, e_rb, e_cc,            \
        (const float *)e_qa, (const float *)e_q1, nE, M, smax, (float2 *)P)
#define NUDIM_COLFS8(R1, R2)                                                                     \
    k_colfft_interp_fs8<R1, R2><<<dim3(nblk, nb), 256, sizeof(float2) * 8 * fs8_gs<R1, R2>(),    \
                                  st>>>((const float2 *)H, N0, n1, (const float2 *)tw0, blk_off, \
                                        ent, e_rb, e_cc, (const float *)e_qa,                   \
                                        (const float *)e_q1, nE, M, smax, (float2 *)P)
            if (sizeof(T) == 4 && BC == 8 && n0 == 1024) NUDIM_COLFS8(32, 32);
            else if (sizeof(T) == 4 && BC == 8 && n0 == 512) NUDIM_COLFS8(32, 16);
            else if (sizeof(T) == 4 && BC == 8 && n0 == 256) NUDIM_COLFS8(16, 16);
            else if (sizeof(T) == 4 && BC == 4 && n0 == 1024) NUDIM_COLFS2(32, 32);
            else if (sizeof(T) == 4 && BC == 4 && n0 == 512) NUDIM_COLFS2(32, 16);
            else if (sizeof(T) == 4 && BC == 4 && n0 == 256) NUDIM_COLFS2(16, 16);
            else if (BC == 4 && n0 == 1024) NUDIM_COLFS(32, 32);
            else if (BC == 4 && n0 == 512) NUDIM_COLFS(32, 16);
            else if (BC == 4 && n0 == 256) NUDIM_COLFS(16, 16);
            else
                k_colfft_interp<T><<<dim3(nblk, nb), thr, smem_col, st>>>(
                    H, N0, n0, logn0, n1, BC, tw0, blk_off, ent, e_rb, e_cc, e_qa, e_q1, nE, M,
                    smax, P);
#undef NUDIM_COLFS
#undef NUDIM_COLFS2
#undef NUDIM_COLFS8
            NUDIM_LAUNCH_CHECK();
        }
        {
            ProfScope ps(ctx, PK_CGVEC, st, nb * c * ((double)smax * M + M));
            dim3 g(interp_blocks(), nb);
            switch (ia.mode) {
            case IM_PLAIN: k_combine<T, IM_PLAIN><<<g, 256, 0, st>>>(P, nslots, M, smax, p0, ia); break;
            case IM_RESID: k_combine<T, IM_RESID><<<g, 256, 0, st>>>(P, nslots, M, smax, p0, ia); break;
            case IM_DOTV: k_combine<T, IM_DOTV><<<g, 256, 0, st>>>(P, nslots, M, smax, p0, ia); break;
            default: k_combine<T, IM_CONSTRAINT><<<g, 256, 0, st>>>(P, nslots, M, smax, p0, ia); break;
            }
            NUDIM_LAUNCH_CHECK();
        }
    }
    return NUDIM_OK;
}

//   spread    tables + nb*c*(M + n0*n1)   node values in, grid out
//   col IFFT  nb*c*(n0*n1 + N0*n1)        grid in, column spectra out
//   row pass  nb*c*(N0*n1 + 2*N0*N1)      column spectra in, coefficients out
template <typename T>
int NfftDev<T>::adjoint_fused(int nplanes, const SpreadArgs<T> &sa, const CropArgs<T> &ca,
                              cudaStream_t st)
{
    if (trafo_only) {
        set_error("NFFT plan built for the trafo only has no adjoint");
        return NUDIM_ESTATE;
    }
    int chunk = fused_chunk(nplanes, (size_t)N0 * n1 + (size_t)n0 * n1 + 32 * (size_t)nextra);
    void *wsv;
    size_t nH = (size_t)N0 * n1 * chunk, nG = (size_t)n0 * n1 * chunk;
    NUDIM_TRY(workspace(sizeof(C) * (nH + nG + 32 * (size_t)nextra * chunk), &wsv));
    C *Hp = (C *)wsv, *G = Hp + nH, *part = G + nG;
    int logn0 = ilog2(n0), logn1 = ilog2(n1);
    const double c = sizeof(C), tab = (double)M * (8 + 2 * kW * sizeof(T));
    for (int p0 = 0; p0 < nplanes; p0 += chunk) {
        int nb = std::min(chunk, nplanes - p0);
        {
            ProfScope ps(ctx, PK_SPREAD, st, tab + nb * c * ((double)M + (double)n0 * n1));
            dim3 g(ceil_div(nunits, kGatherUnitsPerCta), ceil_div(nb, Pa));
            const int thr = 32 * kGatherWarps;
#define NUDIM_GATHER(WT, PP)                                                                    \
    k_spread_gather<T, WT, PP><<<g, thr, smem_spread, st>>>(sa, units, nunits, band_node,       \
                                                            band_w, nbands, n0, n1, BCa, nb,    \
                                                            p0, G, part)
            if (sa.w) {
                if (Pa == 8) NUDIM_GATHER(true, 8);
                else if (Pa == 4) NUDIM_GATHER(true, 4);
                else if (Pa == 2) NUDIM_GATHER(true, 2);
                else NUDIM_GATHER(true, 1);
            } else {
                if (Pa == 8) NUDIM_GATHER(false, 8);
                else if (Pa == 4) NUDIM_GATHER(false, 4);
                else if (Pa == 2) NUDIM_GATHER(false, 2);
                else NUDIM_GATHER(false, 1);
            }
#undef NUDIM_GATHER
            NUDIM_LAUNCH_CHECK();
            if (nfix > 0) {
                k_spread_fixup<T><<<dim3(nfix, ceil_div(nb, 8)), 256, 0, st>>>(
                    fixups, nbands, n0, n1, BCa, nb, part, G);
                NUDIM_LAUNCH_CHECK();
            }
        }
        {
            ProfScope ps(ctx, PK_SPREAD, st, nb * c * ((double)n0 * n1 + (double)N0 * n1));
            const size_t smem_fs =
                sizeof(C) * 4 *
                (n0 == 1024 ? fs_col_stride<32, 32>() : n0 == 512 ? fs_col_stride<32, 16>()
                                                                  : fs_col_stride<16, 16>());
            if (BCa == 4 && n0 == 1024)
                k_colifft_fs<T, 32, 32><<<dim3(nblka, nb), 128, smem_fs, st>>>(G, N0, n1, tw0, Hp);
            else if (BCa == 4 && n0 == 512)
                k_colifft_fs<T, 32, 16><<<dim3(nblka, nb), 64, smem_fs, st>>>(G, N0, n1, tw0, Hp);
            else if (BCa == 4 && n0 == 256)
                k_colifft_fs<T, 16, 16><<<dim3(nblka, nb), 64, smem_fs, st>>>(G, N0, n1, tw0, Hp);
            else
                k_colifft<T><<<dim3(nblka, nb), 256, smem_colifft, st>>>(G, N0, n0, logn0, n1,
                                                                          BCa, tw0, Hp);
            NUDIM_LAUNCH_CHECK();
        }
        {
            ProfScope ps(ctx, PK_CROP, st, nb * c * ((double)N0 * n1 + 2.0 * N0 * N1));
            dim3 g(ceil_div(N0, rows), nb);
#define NUDIM_CROPFS(MD, R1, R2)                                                                 \
    k_rowifft_crop_fs<T, MD, R1, R2><<<g, 128, smem_row, st>>>(Hp, N0, N1, c0, c1, tw1, p0, ca)
#define NUDIM_CROPFS_N(MD)                                                                       \
    do {                                                                                        \
        if (n1 == 1024) NUDIM_CROPFS(MD, 32, 32);                                               \
        else if (n1 == 512) NUDIM_CROPFS(MD, 32, 16);                                           \
        else NUDIM_CROPFS(MD, 16, 16);                                                          \
    } while (0)
            if (row_fs) {
                if (ca.mode == CM_PLAIN) NUDIM_CROPFS_N(CM_PLAIN);
                else if (ca.mode == CM_DOT) NUDIM_CROPFS_N(CM_DOT);
                else NUDIM_CROPFS_N(CM_INIT);
            } else
#undef NUDIM_CROPFS_N
#undef NUDIM_CROPFS
            switch (ca.mode) {
            case CM_PLAIN: k_rowifft_crop<T, CM_PLAIN><<<g, 256, smem_row, st>>>(Hp, N0, N1, n1, logn1, rows, c0, c1, tw1, p0, ca); break;
            case CM_DOT: k_rowifft_crop<T, CM_DOT><<<g, 256, smem_row, st>>>(Hp, N0, N1, n1, logn1, rows, c0, c1, tw1, p0, ca); break;
            default: k_rowifft_crop<T, CM_INIT><<<g, 256, smem_row, st>>>(Hp, N0, N1, n1, logn1, rows, c0, c1, tw1, p0, ca); break;
            }
            NUDIM_LAUNCH_CHECK();
        }
    }
    return NUDIM_OK;
}

template int NfftDev<double>::init_fused(const NfftTables &, cudaStream_t);
template int NfftDev<float>::init_fused(const NfftTables &, cudaStream_t);

// NUDIM_CTX_AUTOTUNE: for a geometry not yet tuned in this context, build the
// fused plan for each trafo column width (4, 2) and planes per spreading
// gather pass (8, 4, 2), time one trafo + adjoint of a batch of planes for each (after one
// untimed pair, CUDA events on the plan's stream), keep the fastest in the
// context and use it for this plan.  Candidates that build the same plan as
// an earlier one are not timed again.
template <typename T> int NfftDev<T>::autotune(const NfftTables &t, cudaStream_t st)
{
    const auto key = std::make_tuple(t.N0, t.N1, t.M, (int)sizeof(T));
    auto hit = ctx->tuned.find(key);
    if (hit != ctx->tuned.end()) {
        tune_bc = hit->second.first;
        tune_planes = hit->second.second;
        return NUDIM_OK;
    }
    const int nb = 16;  // planes per timed transform
    void *fh = nullptr, *f = nullptr;
    const size_t bh = sizeof(C) * (size_t)nb * t.N0 * t.N1, bf = sizeof(C) * (size_t)nb * t.M;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = NUDIM_OK;
    if (cudaMallocAsync(&fh, bh, st) != cudaSuccess || cudaMallocAsync(&f, bf, st) != cudaSuccess ||
        cudaMemsetAsync(fh, 0x3c, bh, st) != cudaSuccess ||
        cudaMemsetAsync(f, 0x3c, bf, st) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        set_error("autotune: device allocation failed");
        rc = NUDIM_ENOMEM;
    }
    float best = 0.f;
    int choice_bc = 0, choice_p = 0;
    std::vector<std::pair<int, int>> built;  // (BC, Pa) of the plans already timed
    for (int bcc : {8, 4, 2})
        for (int pc : {8, 4, 2}) {
            if (rc) break;
            NfftDev<T> trial;
            trial.tune_bc = bcc;
            trial.tune_planes = pc;
            if (trial.init(ctx, t, st, wsp) != NUDIM_OK || !trial.fused) {
                trial.release();
                continue;
            }
            const std::pair<int, int> got(trial.BC, trial.Pa);
            bool seen = false;
            for (auto &b : built) seen = seen || b == got;
            if (!seen) {
                built.push_back(got);
                PadArgs<T> pa;
                pa.src = fh;
                pa.src_stride = (size_t)t.N0 * t.N1;
                InterpArgs<T> ia;
                ia.out = (C *)f;
                ia.out_stride = t.M;
                SpreadArgs<T> sa;
                sa.f = (const C *)f;
                sa.f_stride = t.M;
                CropArgs<T> ca;
                ca.out = (C *)fh;
                ca.out_stride = (size_t)t.N0 * t.N1;
                float ms = 0.f;
                rc = trial.trafo(nb, pa, ia, st);
                if (!rc) rc = trial.adjoint(nb, sa, ca, st);
                if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = NUDIM_ECUDA;
                if (!rc) rc = trial.trafo(nb, pa, ia, st);
                if (!rc) rc = trial.adjoint(nb, sa, ca, st);
                if (!rc && (cudaEventRecord(e1, st) != cudaSuccess ||
                            cudaEventSynchronize(e1) != cudaSuccess ||
                            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                    rc = NUDIM_ECUDA;
                if (!rc && (choice_bc == 0 || ms < best)) {
                    best = ms;
                    choice_bc = bcc;
                    choice_p = pc;
                }
            }
            trial.release();
            if (rc) break;
        }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (fh) cudaFreeAsync(fh, st);
    if (f) cudaFreeAsync(f, st);
    if (rc) return rc;
    if (choice_bc) {
        ctx->tuned[key] = std::make_pair(choice_bc, choice_p);
        tune_bc = choice_bc;
        tune_planes = choice_p;
    }
    return NUDIM_OK;
}

// ================================================================ Toeplitz operator
// K on the circulant in FP64 (k_toep_gtable, k_toep_circ), its nt x nt DFT
// (cuFFT, FP64, once per plan), divided by nt^2 and laid out in the column
// pass's read order in the plan's precision.
template <typename T> int NfftDev<T>::toeplitz_init(const PolarGeom &g, cudaStream_t st)
{
    if (!toeplitz_fits()) {
        set_error("Toeplitz operator: needs the fused four-step path on a square grid of 256, 512 "
                  "or 1024 points");
        return NUDIM_EINVAL;
    }
    if (g.A <= 0 || (size_t)g.A * N1 != (size_t)M || !g.r || !g.sg || !g.cg) {
        set_error("Toeplitz operator: the nodes must be A lines of N1 radii");
        return NUDIM_EINVAL;
    }
    if (toeplitz) return NUDIM_OK;
    const double two_pi = 6.283185307179586;
    // the smallest supported circulant that holds |m| < N without wrap
    // (NUDIM_TOEPLITZ_GRID=nfft keeps the NFFT grid's size)
    const char *eg = getenv("NUDIM_TOEPLITZ_GRID");
    const bool small = !(eg && !strcmp(eg, "nfft"));
    const int nt = (small && 2 * N0 - 1 <= 768 && n0 > 768) ? 768 : n0;
    const size_t nn = (size_t)nt * nt;
    // G's table: |s| <= |m0| + |m1| < N0 + N1
    const double delta = 1.0 / 32;
    const int K0 = (int)std::ceil((N0 + N1) / delta) + 8, Ns = 2 * K0 + 1;
    std::vector<T> hones(std::max(N0, N1), T(1));
    std::vector<C> htw(nt);
    for (int k = 0; k < nt; k++) {
        const double a = -two_pi * (double)k / nt;
        htw[k] = mkc<T>((T)std::cos(a), (T)std::sin(a));
    }
    void *dr = nullptr, *dw = nullptr, *dsg = nullptr, *dcg = nullptr, *dG = nullptr, *dc = nullptr;
    void *d1 = nullptr, *kh = nullptr, *dtw = nullptr;
    // temporaries released stream-ordered after their last use; on failure
    // the kept buffers too
    auto done = [&](int e) {
        for (void *q : {dr, dw, dsg, dcg, dG, dc})
            if (q) cudaFreeAsync(q, st);
        if (e) {
            for (void *q : {d1, kh, dtw})
                if (q) cudaFreeAsync(q, st);
        }
        return e;
    };
    int rc = upload_async(&dr, g.r, sizeof(double) * N1, st);
    if (!rc && g.wr) rc = upload_async(&dw, g.wr, sizeof(double) * N1, st);
    if (!rc) rc = upload_async(&dsg, g.sg, sizeof(double) * g.A, st);
    if (!rc) rc = upload_async(&dcg, g.cg, sizeof(double) * g.A, st);
    if (!rc) rc = upload_async(&d1, hones.data(), sizeof(T) * hones.size(), st);
    if (!rc && nt != n0) rc = upload_async(&dtw, htw.data(), sizeof(C) * htw.size(), st);
    if (rc) return done(rc);
    if (cudaMallocAsync(&dG, sizeof(double2) * Ns, st) != cudaSuccess ||
        cudaMallocAsync(&dc, sizeof(double2) * nn, st) != cudaSuccess ||
        cudaMallocAsync(&kh, sizeof(C) * nn, st) != cudaSuccess) {
        set_error("Toeplitz operator: out of device memory");
        return done(NUDIM_ECUDA);
    }
    k_toep_gtable<<<(unsigned)ceil_div(Ns, 128), 128, 0, st>>>((const double *)dr,
                                                               (const double *)dw, N1, delta, K0,
                                                               Ns, (double2 *)dG);
    ++g_launches;
    k_toep_circ<<<(unsigned)ceil_div((long)(nt / 2 + 1) * nt, 128), 128, 0, st>>>(
        (const double2 *)dG, delta, K0, (const double *)dsg, (const double *)dcg, g.A, N0, N1, nt,
        (double2 *)dc);
    ++g_launches;
    if (cudaGetLastError() != cudaSuccess) {
        set_error("Toeplitz operator: setup kernel launch failed");
        return done(NUDIM_ECUDA);
    }
    cufftHandle h;
    if ((rc = ctx_fft2d(ctx, nt, nt, 1, NUDIM_FP64, &h))) return done(rc);
    if (cufftSetStream(h, st) != CUFFT_SUCCESS) {
        set_error("Toeplitz operator: cufftSetStream failed");
        return done(NUDIM_ECUDA);
    }
    if ((rc = fft_exec<double>(h, (double2 *)dc, CUFFT_FORWARD))) return done(rc);
    // the column pass's four-step split of the circulant's size
    const int R1 = nt == 256 ? 16 : nt == 768 ? 24 : 32, R2 = nt / R1;
    k_toep_layout<T><<<(unsigned)ceil_div((long)nn, 256), 256, 0, st>>>((const double2 *)dc, nt,
                                                                         nt, R1, R2, (C *)kh);
    ++g_launches;
    if (cudaGetLastError() != cudaSuccess) {
        set_error("Toeplitz operator: setup kernel launch failed");
        return done(NUDIM_ECUDA);
    }
    done(NUDIM_OK);
    khat = (C *)kh;
    ones = (T *)d1;
    nT = nt;
    twT = dtw ? (C *)dtw : tw0;
    bytes += sizeof(C) * nn + sizeof(T) * hones.size() + (dtw ? sizeof(C) * nt : 0);
    toeplitz = true;
    return NUDIM_OK;
}

// out = T src over nplanes planes: row FFT of the zero-padded rows (unit
// factors), the column pass, the inverse row FFT with the crop in ca's mode.
// Scratch: one N0 x n1 plane of row spectra per plane of a chunk.
template <typename T>
int NfftDev<T>::toeplitz_apply(int nplanes, const PadArgs<T> &pa, const CropArgs<T> &ca,
                               cudaStream_t st)
{
    if (!toeplitz) {
        set_error("Toeplitz operator not initialised");
        return NUDIM_ESTATE;
    }
    const int nt = nT;
    int chunk = fused_chunk(nplanes, (size_t)N0 * nt);
    void *wsv;
    size_t nH = (size_t)N0 * nt * chunk;
    NUDIM_TRY(workspace(sizeof(C) * nH, &wsv));
    C *H = (C *)wsv;
    const double c = sizeof(C);
    const size_t smem_t =
        sizeof(C) * 4 *
        (nt == 1024  ? fs_col_stride<32, 32>()
         : nt == 768 ? fs_col_stride<24, 32>()
         : nt == 512 ? fs_col_stride<32, 16>()
                     : fs_col_stride<16, 16>());
    const size_t smem_r = nt == 768 ? sizeof(C) * 4 * fs_row_stride<24, 32>() : smem_row;
    const int trows = nt == 768 ? 4 : rows;
    for (int p0 = 0; p0 < nplanes; p0 += chunk) {
        int nb = std::min(chunk, nplanes - p0);
        {
            ProfScope ps(ctx, PK_TOEPLITZ, st, nb * c * ((double)N0 * N1 + (double)N0 * nt));
            dim3 g(ceil_div(N0, trows), nb);
#define NUDIM_TROW(MD, R1, R2)                                                                   \
    k_rowfft_fs<T, MD, R1, R2><<<g, 128, smem_r, st>>>(pa.src, pa.src_stride, N0, N1, ones, ones, \
                                                        twT, p0, H, pa.f_init, pa.f_stride)
            if (pa.mode == PM_COMPLEX) {
                if (nt == 1024) NUDIM_TROW(PM_COMPLEX, 32, 32);
                else if (nt == 768) NUDIM_TROW(PM_COMPLEX, 24, 32);
                else if (nt == 512) NUDIM_TROW(PM_COMPLEX, 32, 16);
                else NUDIM_TROW(PM_COMPLEX, 16, 16);
            } else {
                if (nt == 1024) NUDIM_TROW(PM_REAL_INIT, 32, 32);
                else if (nt == 768) NUDIM_TROW(PM_REAL_INIT, 24, 32);
                else if (nt == 512) NUDIM_TROW(PM_REAL_INIT, 32, 16);
                else NUDIM_TROW(PM_REAL_INIT, 16, 16);
            }
#undef NUDIM_TROW
            NUDIM_LAUNCH_CHECK();
        }
        {
            // H read and written in place; khat (n0 n1 values) read per plane
            ProfScope ps(ctx, PK_TOEPLITZ, st, nb * c * 2.0 * N0 * nt + c * (double)nt * nt);
            if (nt == 1024)
                k_col_toeplitz<T, 32, 32><<<dim3(nt / 4, nb), 128, smem_t, st>>>(H, N0, nt, twT,
                                                                                  khat);
            else if (nt == 768)
                k_col_toeplitz<T, 24, 32><<<dim3(nt / 4, nb), 128, smem_t, st>>>(H, N0, nt, twT,
                                                                                  khat);
            else if (nt == 512)
                k_col_toeplitz<T, 32, 16><<<dim3(nt / 4, nb), 64, smem_t, st>>>(H, N0, nt, twT,
                                                                                 khat);
            else
                k_col_toeplitz<T, 16, 16><<<dim3(nt / 4, nb), 64, smem_t, st>>>(H, N0, nt, twT,
                                                                                 khat);
            NUDIM_LAUNCH_CHECK();
        }
        {
            ProfScope ps(ctx, PK_TOEPLITZ, st, nb * c * ((double)N0 * nt + 2.0 * N0 * N1));
            dim3 g(ceil_div(N0, trows), nb);
#define NUDIM_TCROP(MD, R1, R2)                                                                  \
    k_rowifft_crop_fs<T, MD, R1, R2><<<g, 128, smem_r, st>>>(H, N0, N1, ones, ones, twT, p0, ca)
#define NUDIM_TCROP_N(MD)                                                                        \
    do {                                                                                        \
        if (nt == 1024) NUDIM_TCROP(MD, 32, 32);                                                \
        else if (nt == 768) NUDIM_TCROP(MD, 24, 32);                                            \
        else if (nt == 512) NUDIM_TCROP(MD, 32, 16);                                            \
        else NUDIM_TCROP(MD, 16, 16);                                                           \
    } while (0)
            if (ca.mode == CM_TRESID) NUDIM_TCROP_N(CM_TRESID);
            else if (ca.mode == CM_TPDOT) NUDIM_TCROP_N(CM_TPDOT);
            else NUDIM_TCROP_N(CM_PLAIN);
#undef NUDIM_TCROP_N
#undef NUDIM_TCROP
            NUDIM_LAUNCH_CHECK();
        }
    }
    return NUDIM_OK;
}

template int NfftDev<double>::toeplitz_init(const PolarGeom &, cudaStream_t);
template int NfftDev<float>::toeplitz_init(const PolarGeom &, cudaStream_t);
template int NfftDev<double>::toeplitz_apply(int, const PadArgs<double> &,
                                             const CropArgs<double> &, cudaStream_t);
template int NfftDev<float>::toeplitz_apply(int, const PadArgs<float> &, const CropArgs<float> &,
                                            cudaStream_t);
template int NfftDev<double>::autotune(const NfftTables &, cudaStream_t);
template int NfftDev<float>::autotune(const NfftTables &, cudaStream_t);
template void NfftDev<double>::release_fused();
template void NfftDev<float>::release_fused();
template int NfftDev<double>::fused_chunk(int, size_t) const;
template int NfftDev<float>::fused_chunk(int, size_t) const;
template int NfftDev<double>::trafo_fused(int, const PadArgs<double> &, const InterpArgs<double> &,
                                          cudaStream_t);
template int NfftDev<float>::trafo_fused(int, const PadArgs<float> &, const InterpArgs<float> &,
                                         cudaStream_t);
template int NfftDev<double>::adjoint_fused(int, const SpreadArgs<double> &,
                                            const CropArgs<double> &, cudaStream_t);
template int NfftDev<float>::adjoint_fused(int, const SpreadArgs<float> &,
                                           const CropArgs<float> &, cudaStream_t);

}  // namespace nudim
