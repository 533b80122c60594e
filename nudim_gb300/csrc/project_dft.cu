// project_dft.cu -- the Fourier samples of projection_sim -m DFT
// (src/projection_sim.c:516-560) on the GPU, FP64.
//
// The reference sums, for every node of every tilt, all nx*ny*nz voxels times
// cos(2 PI t) - i sin(2 PI t), t = col X + row Y + slc Z, with the centred
// indices col = x - nx/2, row = y - ny/2, slc = z - nz/2, the 3D equal-angle
// nodes of grid.c:5-57 and PI = 3.1415926 (grid.h:11).  The truncated PI
// makes this differ from the true transform (and from -m 2D1D) by about
// 1e-6 relative, so it is reproduced here: the exponential factors into one
// phase per axis, and the sum is done exactly as three contractions,
//   A[z][y][m] = sum_x D[z][y][x] EX[x][m]          (real x complex, tiled)
//   B[z][m]    = sum_y EY[y][m] A[z][y][m]
//   S[j][m]    = sum_z EZ[z][j] B[z][m]
// with m = tilt * np + radial index (the node's X = r cos g, Y = r sin g) and
// j the node's Z index.  FP64 throughout; GB300's FP64 rate bounds the first
// contraction (2 nx ny nz M fused multiply-adds).
#include <algorithm>

#include "engine.cuh"

namespace nudim {

// E[k][m] = exp(-i 2 PI (k - K/2) c[m])
__global__ void k_dft_phase(const double *__restrict__ c, int K, int Mc, double2 *__restrict__ E)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)K * Mc) return;
    int k = (int)(t / Mc), m = (int)(t % Mc);
    double s, co;
    sincos(2 * kRefPi * ((double)(k - K / 2) * c[m]), &s, &co);
    E[t] = make_double2(co, -s);
}

// A[r][m] = sum_x D[r][x] EX[x][m] for rows r < R of D (nx per row).  64 x 64
// output tiles, 256 threads, each 4 rows x 4 nodes (rows ty + 16 i, nodes
// tx + 16 j), x in steps of 16 through shared memory.
constexpr int kDftT = 64, kDftK = 16;
__global__ void __launch_bounds__(256)
k_dft_x(const double *__restrict__ D, int R, int nx, const double2 *__restrict__ EX, int Mc,
        double2 *__restrict__ A)
{
    __shared__ double sd[kDftK][kDftT + 1];
    __shared__ double2 se[kDftK][kDftT];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int r0 = blockIdx.y * kDftT, m0 = blockIdx.x * kDftT;
    double2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = make_double2(0, 0);
    for (int x0 = 0; x0 < nx; x0 += kDftK) {
        for (int l = threadIdx.x; l < kDftT * kDftK; l += 256) {
            int rr = l / kDftK, xx = l % kDftK, r = r0 + rr, x = x0 + xx;
            sd[xx][rr] = (r < R && x < nx) ? D[(size_t)r * nx + x] : 0.0;
        }
        for (int l = threadIdx.x; l < kDftT * kDftK; l += 256) {
            int xx = l / kDftT, mm = l % kDftT, x = x0 + xx, m = m0 + mm;
            se[xx][mm] = (x < nx && m < Mc) ? EX[(size_t)x * Mc + m] : make_double2(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kDftK; k++) {
            double dv[4];
            double2 ev[4];
#pragma unroll
            for (int i = 0; i < 4; i++) dv[i] = sd[k][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) ev[j] = se[k][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j].x = fma(dv[i], ev[j].x, acc[i][j].x);
                    acc[i][j].y = fma(dv[i], ev[j].y, acc[i][j].y);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int r = r0 + ty + 16 * i, m = m0 + tx + 16 * j;
            if (r < R && m < Mc) A[(size_t)r * Mc + m] = acc[i][j];
        }
}

__device__ __forceinline__ double2 cmul_acc(double2 acc, double2 a, double2 b)
{
    acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
    acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
    return acc;
}

// B[z][m] = sum_y EY[y][m] A[z - z0][y][m] for z in [z0, z0 + nzc)
__global__ void k_dft_y(const double2 *__restrict__ A, const double2 *__restrict__ EY, int ny,
                        int Mc, int z0, double2 *__restrict__ B)
{
    int m = blockIdx.x * blockDim.x + threadIdx.x, zl = blockIdx.y;
    if (m >= Mc) return;
    double2 acc = make_double2(0, 0);
    const double2 *a = A + (size_t)zl * ny * Mc + m;
    for (int y = 0; y < ny; y++) acc = cmul_acc(acc, EY[(size_t)y * Mc + m], a[(size_t)y * Mc]);
    B[(size_t)(z0 + zl) * Mc + m] = acc;
}

// S[j][m] = sum_z EZ[z][j] B[z][m]
__global__ void k_dft_z(const double2 *__restrict__ B, const double2 *__restrict__ EZ, int nz,
                        int Mc, double2 *__restrict__ S)
{
    int m = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (m >= Mc) return;
    double2 acc = make_double2(0, 0);
    for (int z = 0; z < nz; z++) acc = cmul_acc(acc, EZ[(size_t)z * nz + j], B[(size_t)z * Mc + m]);
    S[(size_t)j * Mc + m] = acc;
}

int dft_slices(const double *dens, int nx, int ny, int nz, int np, const double *x2, int ns,
               double2 *S, size_t budget, cudaStream_t st)
{
    const int Mc = ns * np;
    // node coordinates: X = r cos g, Y = r sin g (grid.c:24-25; the 2D table
    // holds (r sin g, r cos g)), Z by repeated addition of 1/nz (grid.c:14-17)
    std::vector<double> cx(Mc), cy(Mc), cz(nz);
    for (int m = 0; m < Mc; m++) {
        cy[m] = x2[2 * (size_t)m + 0];
        cx[m] = x2[2 * (size_t)m + 1];
    }
    double z0 = -0.5 - 1.0 / nz;
    for (int j = 0; j < nz; j++) cz[j] = (z0 += 1.0 / nz);
    double *dc = nullptr;
    double2 *EX = nullptr, *EY = nullptr, *EZ = nullptr, *A = nullptr, *B = nullptr;
    const size_t row_bytes = sizeof(double2) * (size_t)ny * Mc;
    const int nzc = (int)std::max<size_t>(1, std::min<size_t>(nz, budget / row_bytes));
    int rc = NUDIM_OK;
    if (cudaMalloc(&dc, sizeof(double) * (2 * (size_t)Mc + nz)) ||
        cudaMalloc(&EX, sizeof(double2) * (size_t)nx * Mc) ||
        cudaMalloc(&EY, sizeof(double2) * (size_t)ny * Mc) ||
        cudaMalloc(&EZ, sizeof(double2) * (size_t)nz * nz) ||
        cudaMalloc(&A, row_bytes * nzc) || cudaMalloc(&B, sizeof(double2) * (size_t)nz * Mc)) {
        set_error("out of device memory in projection_sim -m DFT");
        rc = NUDIM_ENOMEM;
    }
    if (!rc) {
        cudaMemcpyAsync(dc, cx.data(), sizeof(double) * Mc, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dc + Mc, cy.data(), sizeof(double) * Mc, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dc + 2 * Mc, cz.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, st);
        k_dft_phase<<<ceil_div((long)nx * Mc, 256), 256, 0, st>>>(dc, nx, Mc, EX);
        k_dft_phase<<<ceil_div((long)ny * Mc, 256), 256, 0, st>>>(dc + Mc, ny, Mc, EY);
        k_dft_phase<<<ceil_div((long)nz * nz, 256), 256, 0, st>>>(dc + 2 * Mc, nz, nz, EZ);
        for (int zs = 0; zs < nz && !rc; zs += nzc) {
            int zn = std::min(nzc, nz - zs), R = zn * ny;
            k_dft_x<<<dim3(ceil_div(Mc, kDftT), ceil_div(R, kDftT)), 256, 0, st>>>(
                dens + (size_t)zs * ny * nx, R, nx, EX, Mc, A);
            k_dft_y<<<dim3(ceil_div(Mc, 128), zn), 128, 0, st>>>(A, EY, ny, Mc, zs, B);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) rc = cuda_fail(e, "projection_sim -m DFT", __FILE__, __LINE__);
        }
    }
    if (!rc) {
        k_dft_z<<<dim3(ceil_div(Mc, 128), nz), 128, 0, st>>>(B, EZ, nz, Mc, S);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "projection_sim -m DFT", __FILE__, __LINE__);
    }
    cudaStreamSynchronize(st);
    cudaFree(dc);
    cudaFree(EX);
    cudaFree(EY);
    cudaFree(EZ);
    cudaFree(A);
    cudaFree(B);
    return rc;
}

}  // namespace nudim
