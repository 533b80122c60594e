// engine.cuh -- device engine of the NUDIM reconstruction loop.
//
// Data layout in HBM (per job, precision T = double | float, C = complex T):
//   img_a, img_b   V = nz*np*np reals, [z][y][x]   (current / previous volume)
//   data           V complex, [q][y][x]: Z-frequency planes in FFT order;
//                  doubles as the CGNR solution f of every plane
//   y, r, v        nz*M complex: CGNR right-hand side, residual, A p
//   z, p           V complex: CGNR normal residual and search direction
//   slices         nz*M complex: measured / filled Fourier samples, stored
//                  in the q order of `data` (plane q <-> slice (q+nz/2)%nz)
//   grid workspace chunk*n0*n1 complex, owned by the context
#pragma once

#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "tables.h"

namespace nudim {
// Kernel classes timed by the per-kernel CUDA-event profiler.
enum ProfKernel {
    PK_PAD = 0,     // deconvolve + pad into the oversampled grid
    PK_FFT2D,       // cuFFT oversampled-grid FFT
    PK_INTERP,      // window interpolation (trafo gather) + epilogue
    PK_SPREAD,      // atomic-free spreading gather (adjoint)
    PK_CROP,        // crop + deconvolve (adjoint) + epilogue
    PK_CGVEC,       // CGNR vector updates and dot finishes
    PK_ZFFT,        // cuFFT Z-axis FFT
    PK_VOLUME,      // pack/unpack, HIO/ER constraint, R-factor
    PK_TV,          // TV gradient + update
    PK_DIFFUSION,   // 2D anisotropic diffusion wavefront
    PK_TOEPLITZ,    // CGNR normal operator by Toeplitz embedding (its three passes)
    PK_COUNT
};
struct ProfRec {
    int k;
    cudaEvent_t a, b;
    double bytes;
};
}  // namespace nudim

struct nudim_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // per-kernel event timing (nudim_ctx_profile)
    bool prof_on = false;
    std::vector<nudim::ProfRec> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
    double prof_ms[nudim::PK_COUNT] = {};
    long long prof_n[nudim::PK_COUNT] = {};
    double prof_bytes[nudim::PK_COUNT] = {};
    void *ws = nullptr;          // shared oversampled-grid workspace
    size_t ws_bytes = 0;
    size_t grid_budget = 0;      // bytes a single NFFT pass may use for grids
    size_t fused_budget = 0;     // scratch bytes of one fused NFFT pass over a chunk of planes
    bool use_fused = true;       // NFFT path: fused (default) or cuFFT grid path
    // NUDIM_CTX_AUTOTUNE: the fused plan choice (trafo column width, planes per
    // spreading CTA) found fastest for each (N0, N1, M, element size)
    bool autotune = false;
    std::map<std::tuple<int, int, int, int>, std::pair<int, int>> tuned;
    std::map<std::tuple<int, int, int, int>, cufftHandle> fft2d;  // n0,n1,batch,prec
    std::map<std::tuple<int, int, int, int>, cufftHandle> fftz;   // nz,P2,prec,kind
    double *scratch = nullptr;   // small reduction workspace (operator-level calls)
    size_t scratch_bytes = 0;
};

namespace nudim {

// Stream-ordered scratch owned by one stream (a job or the context): grows
// with cudaFreeAsync/cudaMallocAsync on that stream, never syncs the device.
// Once a CUDA graph has captured launches that use it, the workspace is
// frozen: a later request for more bytes is an error (NUDIM_ESTATE) instead
// of a reallocation that would leave the graph holding a freed address.
struct Workspace {
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t st = nullptr;
    bool frozen = false;
};
int ws_get(Workspace *w, size_t bytes, void **out);
void ws_release(Workspace *w);

// Times the launches issued on `st` while it lives (one record per scope);
// `bytes` is the algorithmic traffic the scope's launches move.
struct ProfScope {
    nudim_ctx *c;
    int k;
    cudaStream_t st;
    double bytes;
    cudaEvent_t a = nullptr;
    ProfScope(nudim_ctx *c_, int k_, cudaStream_t st_, double bytes_);
    ~ProfScope();
};
int prof_collect(nudim_ctx *c);

int ctx_workspace(nudim_ctx *ctx, size_t bytes, void **p);
int upload_async(void **dst, const void *src, size_t nb, cudaStream_t st);
int ctx_scratch(nudim_ctx *ctx, size_t bytes, double **p);
int ctx_fft2d(nudim_ctx *ctx, int n0, int n1, int batch, int prec, cufftHandle *h);

template <typename T> cufftType fft_c2c();
template <> inline cufftType fft_c2c<double>() { return CUFFT_Z2Z; }
template <> inline cufftType fft_c2c<float>() { return CUFFT_C2C; }
template <typename T> int fft_exec(cufftHandle h, cplx_t<T> *io, int dir);

template <typename T> constexpr int prec_of();
template <> constexpr int prec_of<double>() { return NUDIM_FP64; }
template <> constexpr int prec_of<float>() { return NUDIM_MIXED; }

// ------------------------------------------------------------ epilogues
enum PadMode { PM_COMPLEX = 0, PM_REAL_INIT = 1 };
enum InterpMode { IM_PLAIN = 0, IM_RESID = 1, IM_DOTV = 2, IM_CONSTRAINT = 3 };
// CM_TRESID / CM_TPDOT: the Toeplitz normal operator's row pass (no
// deconvolution): z = out - T f, p = z, |z|^2 / q = T p, Re(p^H q)
enum CropMode { CM_PLAIN = 0, CM_DOT = 1, CM_INIT = 2, CM_TRESID = 3, CM_TPDOT = 4 };

template <typename T> struct PadArgs {
    int mode = PM_COMPLEX;
    const void *src = nullptr;     // plane p at src + p*src_stride elements
    size_t src_stride = 0;
    cplx_t<T> *f_init = nullptr;   // PM_REAL_INIT: complex copy of the real input
    size_t f_stride = 0;
};

template <typename T> struct InterpArgs {
    int mode = IM_PLAIN;
    cplx_t<T> *out = nullptr;      // f (PLAIN/DOTV), r (RESID), y (CONSTRAINT)
    size_t out_stride = 0;
    const cplx_t<T> *y = nullptr;  // RESID: r = y - A f
    size_t y_stride = 0;
    const T *w = nullptr;          // DOTV: weights (nullptr = 1)
    const cplx_t<T> *s = nullptr;  // CONSTRAINT: measured samples
    size_t s_stride = 0;
    const int *known = nullptr;    // CONSTRAINT: per polar line
    int line_len = 1;
    double *part = nullptr;        // per-block partial sums, plane p at part + p*part_stride
    int part_stride = 0;
};

template <typename T> struct SpreadArgs {
    const cplx_t<T> *f = nullptr;
    size_t f_stride = 0;
    const T *w = nullptr;          // nullptr: unweighted
};

template <typename T> struct CropArgs {
    int mode = CM_PLAIN;
    cplx_t<T> *out = nullptr;
    size_t out_stride = 0;
    cplx_t<T> *p_out = nullptr;    // CM_INIT / CM_TRESID: search direction p = z
    const cplx_t<T> *pin = nullptr;  // CM_TPDOT: p of p^H q
    double *part = nullptr;
    int part_stride = 0;
};

// The polar node set in factored form for the Toeplitz operator (host
// arrays): node a * N1 + i = r[i] (sg[a], cg[a]), weight wr[i] (nullptr:
// unweighted).
struct PolarGeom {
    int A = 0;
    const double *r = nullptr, *sg = nullptr, *cg = nullptr, *wr = nullptr;
};

// ------------------------------------------------------------ NFFT plan
template <typename T> struct NfftDev {
    using C = cplx_t<T>;
    nudim_ctx *ctx = nullptr;
    Workspace *wsp = nullptr;  // scratch of the owning stream (nullptr: context's)
    cudaStream_t ast = nullptr;  // stream the tables were allocated on
    int N0 = 0, N1 = 0, n0 = 0, n1 = 0, M = 0;
    int ty = 16, tx = 16, nty = 0, ntx = 0;
    int2 *u = nullptr;
    T *psi = nullptr;       // M x 2kW
    T *c0 = nullptr, *c1 = nullptr;
    int *tile_off = nullptr, *tile_nodes = nullptr;
    size_t bytes = 0;

    // fused path (nfft_fused.cu): no oversampled grid in HBM
    bool fused = false;
    int BC = 0, nblk = 0, smax = 0, rows = 4;    // trafo column blocks; rows per row-pass CTA
    bool row_fs = false;                         // row passes as four-step FFTs
    int BCa = 0, nblka = 0, nbands = 0, ntiles = 0;  // adjoint column blocks and tiles
    int nunits = 0, nfix = 0, nextra = 0;  // spreading work units, split tiles, extra ranges
    int4 *units = nullptr, *fixups = nullptr;
    int Pa = 1;                                     // planes per spreading-gather pass
    // caps on the trafo column width and the planes per spreading CTA for
    // init_fused (0: the defaults, or the NUDIM_TUNE_* environment knobs)
    int tune_bc = 0, tune_planes = 0;
    // set before init: build only the trafo's lists (adjoint() then fails)
    bool trafo_only = false;
    size_t smem_col = 0, smem_row = 0, smem_spread = 0, smem_colifft = 0;
    C *tw0 = nullptr, *tw1 = nullptr;
    int *blk_off = nullptr, *ent = nullptr, *band_off = nullptr, *band_node = nullptr;
    T *band_w = nullptr;            // per adjoint tile entry: R row + BCa column weights
    int nE = 0;                     // trafo entries; their records (structure of arrays):
    int *e_rb = nullptr, *e_cc = nullptr;
    T *e_qa = nullptr, *e_q1 = nullptr;
    unsigned char *nslots = nullptr;

    // uploads go on stream st (tables are consumed by later work on st)
    int init(nudim_ctx *c, const NfftTables &t, cudaStream_t st = nullptr,
             Workspace *w = nullptr);
    void release();
    int workspace(size_t bytes, void **p);
    int chunk_for(int nplanes) const;
    int interp_blocks() const { return ceil_div(M, 256); }
    int crop_blocks() const
    {
        return fused ? ceil_div(N0, rows) : ceil_div((long)N0 * N1, 256);
    }
    int trafo(int nplanes, const PadArgs<T> &pa, const InterpArgs<T> &ia, cudaStream_t st);
    int adjoint(int nplanes, const SpreadArgs<T> &sa, const CropArgs<T> &ca, cudaStream_t st);

    // CGNR's normal operator A^H W A by Toeplitz embedding (nfft_fused.cu):
    // khat = the nT x nT DFT of its kernel K[m] = sum_j w_j e^{2 pi i m x_j},
    // |m| < N (computed in FP64), divided by nT^2 and laid out in the column
    // pass's read order;
    // ones: N0 (or N1, the larger) unit deconvolution factors for the row passes
    C *khat = nullptr;
    T *ones = nullptr;
    bool toeplitz = false;
    // the circulant's size: 768 (= 24 x 32) when 2 N - 1 <= 768 < n, else the
    // NFFT grid n; twT: its twiddles e^{-2 pi i k / nT}
    int nT = 0;
    C *twT = nullptr;
    bool toeplitz_fits() const
    {
        return fused && row_fs && N0 == N1 && n0 == n1 && (n0 == 256 || n0 == 512 || n0 == 1024);
    }
    int toeplitz_init(const PolarGeom &g, cudaStream_t st);
    // out = T src for nplanes planes of N0 x N1 (the row pass in ca's mode;
    // pa as for trafo: PM_COMPLEX or PM_REAL_INIT)
    int toeplitz_apply(int nplanes, const PadArgs<T> &pa, const CropArgs<T> &ca, cudaStream_t st);
    int init_fused(const NfftTables &t, cudaStream_t st);
    int autotune(const NfftTables &t, cudaStream_t st);
    void release_fused();
    int fused_chunk(int nplanes, size_t per_plane) const;
    int trafo_fused(int nplanes, const PadArgs<T> &pa, const InterpArgs<T> &ia, cudaStream_t st);
    int adjoint_fused(int nplanes, const SpreadArgs<T> &sa, const CropArgs<T> &ca,
                      cudaStream_t st);
};


// CGNR over `nplanes` planes (solver_before_loop + iters x loop_one_step).
// f: planes of N0*N1 (start value in, result out), y/r/v: planes of M,
// z/p: planes of N0*N1.  f_zero: the start value is zero (skips A f).
// f_real: when non-null the start value is this real array (planes of
// N0*N1) and f is overwritten with it first.
// q: planes of N0*N1 for T p; with it and a plan whose Toeplitz operator is
// ready, the CG runs in coefficient space (z' = z - alpha T p, v^H W v =
// p^H T p: the same iterates as CGNR in exact arithmetic).
template <typename T> struct CgnrBuffers {
    cplx_t<T> *r = nullptr, *v = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
    double *part = nullptr;   // nplanes * part_stride
    int part_stride = 0;
    double *dots = nullptr;   // nplanes * 4
};

template <typename T>
int cgnr_run(NfftDev<T> &pl, int nplanes, const cplx_t<T> *y, const T *w, cplx_t<T> *f,
             const T *f_real, bool f_zero, int iters, CgnrBuffers<T> &b, cudaStream_t st);

int cgnr_part_stride(int M, int N);

// The serving loop's step (api.cu): queue the job's next outer iteration
// unless it waits on a residual check whose result has not reached the host
// (*issued = false then); never blocks the host.
int job_try_step(nudim_job *jb, bool *issued);

// ------------------------------------------------------------ volume ops
template <typename T>
int launch_pack(const T *img, cplx_t<T> *data, int nz, size_t P2, cudaStream_t st);
template <typename T>
int launch_unpack(const cplx_t<T> *data, T *img, int nz, size_t P2, cudaStream_t st);
template <typename T>
int launch_constraint(T *img, const T *img_last, int nz, int np, int nx, const int *it,
                      int nhio, int height, int ylo, int yhi, cudaStream_t st);
template <typename T>
int launch_finish_r(const double *part, int nparts, int nplanes, int stride, double *rh,
                    const int *it, cudaStream_t st);
int launch_set_counter(int *it, int v, cudaStream_t st);
template <typename T>
int launch_real_to(const double *src, T *dst, size_t n, cudaStream_t st);
template <typename T>
int launch_to_double(const T *src, double *dst, size_t n, cudaStream_t st);

// ------------------------------------------------------------ denoise
// TV-discrete, niter iterations on u in place.  scal: 4 doubles.  With u2 and
// g2 (two more volumes, not aliasing u or grad) each iteration after the
// first is one fused pass (the update folded into the next gradient).
template <typename T>
int tv_run(T *u, T *grad, double *part, int part_cap, double *scal, int nz, int ny, int nx,
           float lam, int niter, int height, int ylo, int yhi, cudaStream_t st,
           T *u2 = nullptr, T *g2 = nullptr);
int tv_part_count(int nz, int ny, int nx);
// projection_sim -m DFT Fourier samples: dens [nz][ny][nx] (device, FP64),
// x2 the 2D equal-angle nodes (host, (r sin g, r cos g) per node, ns*np of
// them) -> S [nz][ns*np] (device); scratch of the X contraction <= budget.
int dft_slices(const double *dens, int nx, int ny, int nz, int np, const double *x2, int ns,
               double2 *S, size_t budget, cudaStream_t st);
template <typename T>
int diffusion_run(T *u, int nz, int ny, int nx, int nx_bound, float lambda, float kappa,
                  int niter, cudaStream_t st);

}  // namespace nudim
