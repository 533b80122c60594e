// api.cu -- the C ABI (include/nudim.h): context, jobs and operator-level
// entry points, plus the job pipeline that replaces
// src/reconstruction.c:304-719 with every Z-plane resident on one GPU.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "engine.cuh"

namespace nudim {
const char *last_error();

// ================================================================ setup kernels
// reconstruction.c:345-355: f_hat[x*nz + z] = proj[z][x] (real, imaginary 0)
__global__ void k_proj_fhat(const double *__restrict__ proj, double2 *__restrict__ fh, int nx,
                            int nz)
{
    int t = blockIdx.y;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx * nz) return;
    int col = i % nx, row = i / nx;
    fh[(size_t)t * nx * nz + (size_t)col * nz + row] =
        make_double2(proj[(size_t)t * nx * nz + i], 0.0);
}

// reconstruction.c:437-484 in the q order of the Z-frequency volume:
// plane q holds slice j = (q + nz/2) % nz.
template <typename T>
__global__ void k_build_slices(const double2 *__restrict__ tomo, const int *__restrict__ known,
                               const int *__restrict__ order, const int *__restrict__ unk_rank,
                               const double *__restrict__ fill, int n_unk_row, int np, int nz,
                               int M, cplx_t<T> *__restrict__ slices)
{
    int q = blockIdx.y;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    int j = (q + nz / 2) % nz;
    int a = i / np, r = i - a * np;
    double re = 0, im = 0;
    if (known[a]) {
        double2 v = tomo[(size_t)order[a] * np * nz + (size_t)j * np + r];
        re = v.x;
        im = v.y;
    } else if (fill) {
        re = fill[(size_t)j * n_unk_row + unk_rank[i]];
    }
    slices[(size_t)q * M + i] = mkc<T>((T)re, (T)im);
}

__global__ void k_real_cplx(const double *__restrict__ d, double2 *__restrict__ c, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) c[i] = make_double2(d[i], 0.0);
}

// projection_sim.c:344-366: slice_t[row][col] = NFFT of plane j = (row+nz/2)%nz
// at radius (col+np/2)%np; plane j's NFFT is row `row` of tmp (q order).
// zshift = nz/2: the 3D/DFT methods' shift of both axes (:470-476, :562-574),
// tmp row j holding the nodes of Z index j.
__global__ void k_sim_gather(const double2 *__restrict__ tmp, double2 *__restrict__ sl, int nz,
                             int np, int M, int zshift)
{
    int t = blockIdx.y;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nz * np) return;
    int row = i / np, col = i - row * np;
    sl[(size_t)t * nz * np + i] =
        tmp[(size_t)((row + zshift) % nz) * M + (size_t)t * np + (col + np / 2) % np];
}

// projection_sim.c:377-390: radial fftshift, real part (zshift = nz/2: the
// 3D/DFT methods' shift of both axes, :482-494, :582-594)
__global__ void k_sim_shift(const double2 *__restrict__ sl, double *__restrict__ out, int nz,
                            int np, int zshift)
{
    int t = blockIdx.y;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nz * np) return;
    int row = i / np, col = i - row * np;
    out[(size_t)t * nz * np + i] =
        sl[(size_t)t * nz * np + (size_t)((row + zshift) % nz) * np + (col + np / 2) % np].x;
}

// ================================================================ per-precision state
template <typename T> struct JobState {
    using C = cplx_t<T>;
    bool live = false;
    NfftDev<T> pl;
    T *img_a = nullptr, *img_b = nullptr, *grad = nullptr, *w = nullptr;
    C *data = nullptr, *y = nullptr, *r = nullptr, *v = nullptr, *z = nullptr, *p = nullptr,
      *q = nullptr, *slices = nullptr;
    int *known = nullptr;
    double *part = nullptr, *dots = nullptr, *tv_part = nullptr, *tv_scal = nullptr,
           *rh = nullptr;
    int part_stride = 0, tv_cap = 0;
    size_t bytes = 0;
    std::vector<void *> owned;
    cudaStream_t st = nullptr;  // the job's stream: every allocation is ordered on it
    cufftHandle zplan = 0;      // Z-axis FFT plan with its work area in zws
    Workspace zws;
    // NFFT scratch of this state alone: the state's captured graph holds its
    // address, so no other state (a mixed job's FP64 corrective state) may
    // regrow it
    Workspace ws;
    int *it = nullptr;          // device copy of the outer-iteration index
    cudaGraphExec_t gexec = nullptr;  // replay of one outer iteration
    bool graph_tried = false;
    unsigned long long graph_kernels = 0;

    template <typename P> int alloc(P **ptr, size_t n)
    {
        size_t b = sizeof(P) * (n ? n : 1);
        void *q = nullptr;
        NUDIM_CUDA(cudaMallocAsync(&q, b, st));
        owned.push_back(q);
        bytes += b;
        *ptr = (P *)q;
        return NUDIM_OK;
    }
    void release()
    {
        for (void *q : owned) cudaFreeAsync(q, st);
        owned.clear();
        pl.release();
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        graph_tried = false;
        if (zplan) cufftDestroy(zplan);
        zplan = 0;
        ws_release(&zws);
        ws_release(&ws);
        live = false;
    }
};

}  // namespace nudim

using namespace nudim;

struct nudim_job {
    nudim_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;  // own stream: jobs overlap on the device
    Workspace ws;                   // NFFT scratch of this job
    nudim_job_desc d{};
    int A = 0, M = 0, nmeas = 0, n_unk_row = 0;
    double pad_min = 0, pad_max = 0;
    NfftTables tabs;
    std::vector<int> known, order, unk_rank;
    std::vector<double> fill;
    bool fill_set = false, ready = false;
    int done = 0;
    JobState<double> s64;
    JobState<float> s32;
    int dump_nn = -1;
    double *dump_before = nullptr, *dump_after = nullptr;
    // the initial volume (reconstruction.c:521-540, recovered-0.txt) kept on
    // the device in the job's precision; sent to the host only on request
    void *vol0 = nullptr;
    int corrections = 0;  // corrective FP64 iterations run
    // periodic FP64 residual check (correct_every with NUDIM_CORRECT_TOL > 0):
    // R of the current volume in FP64 and FP32 land in check_host (pinned) and
    // check_ev marks their arrival; the iteration it decides waits until then
    bool check_pending = false;
    cudaEvent_t check_ev = nullptr;
    double *check_host = nullptr;
    // a mixed job whose last iteration ran in FP64: the FP64 state's volume is
    // the current one (the FP32 copy is refreshed before an FP32 iteration),
    // so consecutive FP64 iterations never round the volume to FP32
    bool fp64_owns = false;
};

struct nudim_nfft_plan {
    nudim_ctx *ctx = nullptr;
    int prec = NUDIM_FP64;
    NfftDev<double> d64;
    NfftDev<float> d32;
    // CGNR scratch, grown on demand
    void *cg = nullptr;
    size_t cg_bytes = 0;
};

namespace nudim {

// ================================================================ Z-FFT
// fftw_plan_many_dft(1, &nz, np*np, data, NULL, np*np, 1, ...)
// (reconstruction.c:556): one plan per job state, its work area allocated
// stream-ordered so that plan creation never synchronises the device.
template <typename T> static int zfft_plan(nudim_job *jb, JobState<T> &s)
{
    if (s.zplan) return NUDIM_OK;
    int P2 = jb->d.np * jb->d.np;
    int n[1] = {jb->d.nz};
    size_t work = 0;
    cufftHandle p;
    NUDIM_CUFFT(cufftCreate(&p));
    NUDIM_CUFFT(cufftSetAutoAllocation(p, 0));
    NUDIM_CUFFT(cufftMakePlanMany(p, 1, n, n, P2, 1, n, P2, 1, fft_c2c<T>(), P2, &work));
    void *wa = nullptr;
    s.zws.st = s.st;
    NUDIM_TRY(ws_get(&s.zws, work ? work : 256, &wa));
    NUDIM_CUFFT(cufftSetWorkArea(p, wa));
    NUDIM_CUFFT(cufftSetStream(p, s.st));
    s.zplan = p;
    return NUDIM_OK;
}

template <typename T> static int zfft(nudim_job *jb, JobState<T> &s, int dir)
{
    NUDIM_TRY(zfft_plan<T>(jb, s));
    int P2 = jb->d.np * jb->d.np;
    ProfScope ps(jb->ctx, PK_ZFFT, s.st, 2.0 * sizeof(cplx_t<T>) * (double)P2 * jb->d.nz);
    return fft_exec<T>(s.zplan, s.data, dir);
}

// ================================================================ job state setup
// The CGNR form of a job state: NFFT (a trafo and an adjoint per step, the
// reference's own route and the FP64 default) or Toeplitz (one convolution
// pass per step, the FP32 default where the plan's grid allows it);
// NUDIM_CG=nfft|toeplitz selects one.  Read when the state is set up.
template <typename T> static bool use_toeplitz(const NfftDev<T> &pl)
{
    if (!pl.toeplitz_fits()) return false;
    const char *e = getenv("NUDIM_CG");
    if (e && !strcmp(e, "nfft")) return false;
    if (e && !strcmp(e, "toeplitz")) return true;
    return sizeof(T) == 4;
}

template <typename T> static int state_init(nudim_job *jb, JobState<T> &s)
{
    if (s.live) return NUDIM_OK;
    int nz = jb->d.nz, np = jb->d.np, M = jb->M;
    size_t P2 = (size_t)np * np, V = P2 * nz;
    s.st = jb->stream;
    s.ws.st = jb->stream;
    NUDIM_TRY(s.pl.init(jb->ctx, jb->tabs, jb->stream, &s.ws));
    s.bytes += s.pl.bytes;
    NUDIM_TRY(s.alloc(&s.img_a, V));
    NUDIM_TRY(s.alloc(&s.img_b, V));
    NUDIM_TRY(s.alloc(&s.data, V));
    NUDIM_TRY(s.alloc(&s.z, V));
    NUDIM_TRY(s.alloc(&s.p, V));
    NUDIM_TRY(s.alloc(&s.y, (size_t)nz * M));
    NUDIM_TRY(s.alloc(&s.r, (size_t)nz * M));
    NUDIM_TRY(s.alloc(&s.v, (size_t)nz * M));
    NUDIM_TRY(s.alloc(&s.slices, (size_t)nz * M));
    NUDIM_TRY(s.alloc(&s.known, jb->A));
    NUDIM_CUDA(cudaMemcpyAsync(s.known, jb->known.data(), sizeof(int) * jb->A,
                               cudaMemcpyHostToDevice, jb->stream));
    if (jb->d.weight) {
        std::vector<double> wd(M);
        cgnr_weights(jb->A, np, jb->d.padangle, wd.data());
        std::vector<T> wt(wd.begin(), wd.end());
        NUDIM_TRY(s.alloc(&s.w, M));
        NUDIM_CUDA(cudaMemcpyAsync(s.w, wt.data(), sizeof(T) * M, cudaMemcpyHostToDevice,
                                   jb->stream));
    }
    if (use_toeplitz<T>(s.pl)) {
        // CGNR's normal operator by Toeplitz embedding: T p into q; its kernel
        // from the polar set's factors and the radial weights (the same for
        // every line), in FP64
        NUDIM_TRY(s.alloc(&s.q, V));
        std::vector<double> r(np), sg(jb->A), cg(jb->A), wall, wr;
        polar_factors(jb->pad_min, jb->pad_max, jb->d.padangle, np, r.data(), sg.data(),
                      cg.data());
        if (jb->d.weight) {
            wall.resize((size_t)M);
            cgnr_weights(jb->A, np, jb->d.padangle, wall.data());
            wr.assign(wall.begin(), wall.begin() + np);
        }
        PolarGeom g;
        g.A = jb->A;
        g.r = r.data();
        g.sg = sg.data();
        g.cg = cg.data();
        g.wr = jb->d.weight ? wr.data() : nullptr;
        NUDIM_TRY(s.pl.toeplitz_init(g, jb->stream));
        s.bytes += (size_t)s.pl.nT * s.pl.nT * sizeof(cplx_t<T>);
    }
    if (jb->d.denoise == NUDIM_DENOISE_TV) {
        NUDIM_TRY(s.alloc(&s.grad, V));
        s.tv_cap = tv_part_count(nz, np, np);
        NUDIM_TRY(s.alloc(&s.tv_part, s.tv_cap));
        NUDIM_TRY(s.alloc(&s.tv_scal, 4));
    }
    s.part_stride = cgnr_part_stride(M, (int)P2);
    NUDIM_TRY(s.alloc(&s.part, (size_t)nz * s.part_stride + 2 * (size_t)nz + 2));
    NUDIM_TRY(s.alloc(&s.dots, (size_t)nz * 4));
    NUDIM_TRY(s.alloc(&s.rh, (size_t)std::max(1, jb->d.nhio + jb->d.ner)));
    NUDIM_TRY(s.alloc(&s.it, 1));
    s.live = true;
    return NUDIM_OK;
}

template <typename T> static CgnrBuffers<T> cg_bufs(JobState<T> &s)
{
    CgnrBuffers<T> b;
    b.r = s.r;
    b.v = s.v;
    b.z = s.z;
    b.p = s.p;
    b.q = s.q;
    b.part = s.part;
    b.part_stride = s.part_stride;
    b.dots = s.dots;
    return b;
}

static int iters_of(const nudim_job *jb) { return jb->d.cgnr_iters > 0 ? jb->d.cgnr_iters : kCgnrIters; }

// Slices, initial inverse NFFT and backward Z-FFT for state s.
template <typename T>
// inverse = false: only the measured samples (the FP64 state of a mixed job
// with correction, whose volume is taken from the FP32 state before each
// corrective iteration)
static int state_setup(nudim_job *jb, JobState<T> &s, const double2 *tomo, const int *d_order,
                       const int *d_rank, const double *d_fill, bool inverse = true)
{
    cudaStream_t st = jb->stream;
    int nz = jb->d.nz, np = jb->d.np, M = jb->M;
    size_t P2 = (size_t)np * np;
    k_build_slices<T><<<dim3(ceil_div(M, 256), nz), 256, 0, st>>>(
        tomo, s.known, d_order, d_rank, d_fill, jb->n_unk_row, np, nz, M, s.slices);
    NUDIM_LAUNCH_CHECK();
    if (!inverse) return NUDIM_OK;
    // reconstruction.c:495-518: f = 0, before_loop + 10 steps, per plane
    CgnrBuffers<T> b = cg_bufs(s);
    NUDIM_TRY(cgnr_run<T>(s.pl, nz, s.slices, s.w, s.data, nullptr, true, iters_of(jb), b, st));
    // :521-540 backward Z-FFT, img[(j + nz/2) % nz] = Re(data[j]) / nz
    NUDIM_TRY(zfft<T>(jb, s, CUFFT_INVERSE));
    NUDIM_TRY(launch_unpack<T>(s.data, s.img_a, nz, P2, st));
    return NUDIM_OK;
}

// One outer HIO/ER iteration nn (reconstruction.c:545-703) on state s.
// One outer iteration.  Every iteration-dependent value (the R-factor slot,
// HIO or ER) is read from the device counter s.it, so the same launch
// sequence can be captured once and replayed (dump = the reference's
// grad_before/grad_after capture, which copies to the host mid-iteration).
template <typename T> static int iterate_body(nudim_job *jb, JobState<T> &s, bool dump)
{
    cudaStream_t st = jb->stream;
    const nudim_job_desc &d = jb->d;
    int nz = d.nz, np = d.np, M = jb->M;
    size_t P2 = (size_t)np * np, V = P2 * nz;
    // :548-559 data[t] = img[(t+nz/2)%nz]; forward Z-FFT
    const double sT = sizeof(T), sC = sizeof(cplx_t<T>);
    {
        ProfScope ps(jb->ctx, PK_VOLUME, st, (sT + sC) * (double)V);
        NUDIM_TRY(launch_pack<T>(s.img_a, s.data, nz, P2, st));
    }
    NUDIM_TRY(zfft<T>(jb, s, CUFFT_FORWARD));
    // :565-582 per plane: trafo, reciprocal constraint, R-factor partials
    PadArgs<T> pa;
    pa.src = s.data;
    pa.src_stride = P2;
    InterpArgs<T> ia;
    ia.mode = IM_CONSTRAINT;
    ia.out = s.y;
    ia.out_stride = M;
    ia.s = s.slices;
    ia.s_stride = M;
    ia.known = s.known;
    ia.line_len = np;
    ia.part = s.part;
    ia.part_stride = s.part_stride;
    NUDIM_TRY(s.pl.trafo(nz, pa, ia, st));
    NUDIM_TRY(launch_finish_r<T>(s.part, s.pl.interp_blocks(), nz, s.part_stride, s.rh, s.it, st));
    // :587-599 warm start from the real-space plane, CGNR, write back
    CgnrBuffers<T> b = cg_bufs(s);
    NUDIM_TRY(cgnr_run<T>(s.pl, nz, s.y, s.w, s.data, s.img_a, false, iters_of(jb), b, st));
    // :607-621 backward Z-FFT, img = Re(shifted data)/nz
    NUDIM_TRY(zfft<T>(jb, s, CUFFT_INVERSE));
    {
        ProfScope ps(jb->ctx, PK_VOLUME, st, (sT + sC) * (double)V);
        NUDIM_TRY(launch_unpack<T>(s.data, s.img_b, nz, P2, st));
    }
    // :624-669 denoise
    if (dump) {
        NUDIM_TRY(launch_to_double<T>(s.img_b, (double *)s.z, V, st));
        NUDIM_CUDA(cudaMemcpyAsync(jb->dump_before, s.z, sizeof(double) * V,
                                   cudaMemcpyDeviceToHost, st));
        NUDIM_CUDA(cudaStreamSynchronize(st));
    }
    if (d.denoise == NUDIM_DENOISE_DIFFUSION) {
        float lam = d.variant == NUDIM_VARIANT_PARALLEL ? 0.4f : 0.25f;
        ProfScope ps(jb->ctx, PK_DIFFUSION, st, 2.0 * sT * (double)V);
        NUDIM_TRY(diffusion_run<T>(s.img_b, nz, np, np, nz, lam, 0.005f, 80, st));
    } else if (d.denoise == NUDIM_DENOISE_TV) {
        bool h = d.height && d.variant == NUDIM_VARIANT_SERIAL;
        int ylo = (2 * d.ncenter - d.nheight) / 2, yhi = (2 * d.ncenter + d.nheight) / 2;
        ProfScope ps(jb->ctx, PK_TV, st, 40 * 5.0 * sT * (double)V);
        // the CGNR vector z (V complex values, rewritten by every CGNR run) is
        // free here: the fused TV passes' second volume and gradient
        T *tv2 = reinterpret_cast<T *>(s.z);
        NUDIM_TRY(tv_run<T>(s.img_b, s.grad, s.tv_part, s.tv_cap, s.tv_scal, nz, np, np, 0.2f, 40,
                            h ? 1 : 0, ylo, yhi, st, tv2, tv2 + V));
    }
    if (dump) {
        NUDIM_TRY(launch_to_double<T>(s.img_b, (double *)s.z, V, st));
        NUDIM_CUDA(cudaMemcpyAsync(jb->dump_after, s.z, sizeof(double) * V,
                                   cudaMemcpyDeviceToHost, st));
        NUDIM_CUDA(cudaStreamSynchronize(st));
    }
    // :672-700 HIO/ER (result lands in img_a: the next img and img_last)
    int ylo, yhi;
    if (d.variant == NUDIM_VARIANT_PARALLEL) {
        ylo = (np - d.nheight) / 2;
        yhi = (np + d.nheight) / 2;
    } else {
        ylo = (2 * d.ncenter - d.nheight) / 2;
        yhi = (2 * d.ncenter + d.nheight) / 2;
    }
    ProfScope ps(jb->ctx, PK_VOLUME, st, 3.0 * sT * (double)V);
    NUDIM_TRY(launch_constraint<T>(s.img_b, s.img_a, nz, np, d.nx, s.it, d.nhio,
                                   d.height ? 1 : 0, ylo, yhi, st));
    return NUDIM_OK;
}

static bool graphs_enabled()
{
    const char *e = getenv("NUDIM_GRAPHS");
    return !(e && e[0] == '0');
}

// Outer iteration nn (reconstruction.c:545-703).  The first eager run sizes
// every workspace and plan; later iterations replay a CUDA graph of the
// same launch sequence (not while profiling or dumping).
template <typename T> static int state_iterate(nudim_job *jb, JobState<T> &s, int nn)
{
    cudaStream_t st = jb->stream;
    bool dump = (nn == jb->dump_nn) && jb->dump_before && jb->d.denoise != NUDIM_DENOISE_NONE;
    NUDIM_TRY(launch_set_counter(s.it, nn, st));
    bool replay = graphs_enabled() && !dump && !jb->ctx->prof_on;
    if (replay && s.gexec) {
        NUDIM_CUDA(cudaGraphLaunch(s.gexec, st));
        g_launches += s.graph_kernels;  // the library's kernels inside the graph
        return NUDIM_OK;
    }
    NUDIM_TRY(iterate_body<T>(jb, s, dump));
    if (replay && !s.graph_tried) {
        s.graph_tried = true;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return NUDIM_OK;
        }
        unsigned long long n0 = g_launches;
        int rc = iterate_body<T>(jb, s, false);
        s.graph_kernels = g_launches - n0;  // captured, not executed
        g_launches = n0;
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc == NUDIM_OK && e == cudaSuccess && g &&
            cudaGraphInstantiate(&s.gexec, g, 0) != cudaSuccess)
            s.gexec = nullptr;
        if (s.gexec) {
            // the graph holds the scratch addresses: they must not move
            s.ws.frozen = true;
            s.zws.frozen = true;
        }
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();  // a failed capture leaves eager execution in place
    }
    return NUDIM_OK;
}

// The measured-slice mismatch R of the state's current volume (the first
// steps of an iteration: pack, forward Z-FFT, trafo with the constraint
// epilogue, reconstruction.c:548-582); R lands in rh[nn], which the iteration
// that follows rewrites.
template <typename T> static int state_residual(nudim_job *jb, JobState<T> &s, int nn)
{
    cudaStream_t st = jb->stream;
    const nudim_job_desc &d = jb->d;
    const int nz = d.nz, np = d.np, M = jb->M;
    const size_t P2 = (size_t)np * np;
    NUDIM_TRY(launch_set_counter(s.it, nn, st));
    NUDIM_TRY(launch_pack<T>(s.img_a, s.data, nz, P2, st));
    NUDIM_TRY(zfft<T>(jb, s, CUFFT_FORWARD));
    PadArgs<T> pa;
    pa.src = s.data;
    pa.src_stride = P2;
    InterpArgs<T> ia;
    ia.mode = IM_CONSTRAINT;
    ia.out = s.y;
    ia.out_stride = M;
    ia.s = s.slices;
    ia.s_stride = M;
    ia.known = s.known;
    ia.line_len = np;
    ia.part = s.part;
    ia.part_stride = s.part_stride;
    NUDIM_TRY(s.pl.trafo(nz, pa, ia, st));
    return launch_finish_r<T>(s.part, s.pl.interp_blocks(), nz, s.part_stride, s.rh, s.it, st);
}

// NUDIM_CORRECT_TOL: relative difference between the FP32 and the FP64 R of
// the current volume above which the periodic check runs the corrective FP64
// iteration; 0 (the default) runs it at every check.
static double correct_tol()
{
    const char *e = getenv("NUDIM_CORRECT_TOL");
    double v = e ? atof(e) : 0.0;
    return v > 0 ? v : 0.0;
}

// The periodic FP64 residual check of a mixed job, queued on the job's
// stream: R of the current volume in both forms, copied to check_host, with
// check_ev recorded after the copies.  Nothing here waits on the host.
static int residual_issue(nudim_job *jb, int nn)
{
    cudaStream_t st = jb->stream;
    size_t V = (size_t)jb->d.np * jb->d.np * jb->d.nz;
    if (jb->fp64_owns) NUDIM_TRY(launch_real_to<float>(jb->s64.img_a, jb->s32.img_a, V, st));
    else NUDIM_TRY(launch_to_double<float>(jb->s32.img_a, jb->s64.img_a, V, st));
    NUDIM_TRY(state_residual<double>(jb, jb->s64, nn));
    NUDIM_TRY(state_residual<float>(jb, jb->s32, nn));
    NUDIM_CUDA(cudaMemcpyAsync(jb->check_host, jb->s64.rh + nn, sizeof(double),
                               cudaMemcpyDeviceToHost, st));
    NUDIM_CUDA(cudaMemcpyAsync(jb->check_host + 1, jb->s32.rh + nn, sizeof(double),
                               cudaMemcpyDeviceToHost, st));
    NUDIM_CUDA(cudaEventRecord(jb->check_ev, st));
    return NUDIM_OK;
}

// FP64 buffers of a mixed job take over from FP32 for one corrective
// iteration: the FP32 volume is widened (unless the previous iteration was
// FP64 too), the iteration runs in FP64 and its R lands in the FP32 history.
static int corrective_iteration(nudim_job *jb, int nn)
{
    cudaStream_t st = jb->stream;
    size_t V = (size_t)jb->d.np * jb->d.np * jb->d.nz;
    if (!jb->fp64_owns) NUDIM_TRY(launch_to_double<float>(jb->s32.img_a, jb->s64.img_a, V, st));
    NUDIM_TRY(state_iterate<double>(jb, jb->s64, nn));
    jb->fp64_owns = true;
    // keep the FP32 R history complete
    NUDIM_CUDA(cudaMemcpyAsync(jb->s32.rh + nn, jb->s64.rh + nn, sizeof(double),
                               cudaMemcpyDeviceToDevice, st));
    return NUDIM_OK;
}

// An FP32 iteration of a mixed job, from the FP64 volume when the previous
// iteration was FP64.
static int mixed_iteration(nudim_job *jb, int nn)
{
    if (jb->fp64_owns) {
        size_t V = (size_t)jb->d.np * jb->d.np * jb->d.nz;
        NUDIM_TRY(launch_real_to<float>(jb->s64.img_a, jb->s32.img_a, V, jb->stream));
        jb->fp64_owns = false;
    }
    return state_iterate<float>(jb, jb->s32, nn);
}

// Which iterations of a mixed job run in FP64: correct_every = k > 0, every
// k-th (subject to the residual check); k < 0, every HIO iteration (nn < nhio).
static bool fp64_iteration(const nudim_job *jb, int nn)
{
    const int k = jb->d.correct_every;
    return k > 0 ? (nn + 1) % k == 0 : k < 0 ? nn < jb->d.nhio : false;
}

// Queue outer iteration jb->done of a job that has one left.  A mixed job's
// check iteration (every correct_every-th, with NUDIM_CORRECT_TOL > 0) first
// queues the residual check; the iteration itself is queued once its result
// is on the host: with block, after waiting for it; without, only if it has
// arrived (*issued = false otherwise, and a later call decides).
static int job_advance(nudim_job *jb, bool block, bool *issued)
{
    *issued = false;
    if (jb->done >= jb->d.nhio + jb->d.ner) return NUDIM_OK;
    const int nn = jb->done;
    if (jb->d.precision == NUDIM_FP64) {
        NUDIM_TRY(state_iterate<double>(jb, jb->s64, nn));
    } else if (fp64_iteration(jb, nn)) {
        const double tol = jb->d.correct_every > 0 ? correct_tol() : 0.0;
        bool need = true;
        if (tol > 0) {
            if (!jb->check_pending) {
                NUDIM_TRY(residual_issue(jb, nn));
                jb->check_pending = true;
            }
            cudaError_t q = block ? cudaEventSynchronize(jb->check_ev) : cudaEventQuery(jb->check_ev);
            if (q == cudaErrorNotReady) return NUDIM_OK;
            if (q != cudaSuccess) return cuda_fail(q, "residual check", __FILE__, __LINE__);
            jb->check_pending = false;
            const double r64 = jb->check_host[0], r32 = jb->check_host[1];
            need = !(fabs(r32 - r64) <= tol * fabs(r64));
        }
        if (need) {
            NUDIM_TRY(corrective_iteration(jb, nn));
            jb->corrections++;
        } else {
            NUDIM_TRY(mixed_iteration(jb, nn));
        }
    } else {
        NUDIM_TRY(mixed_iteration(jb, nn));
    }
    jb->done++;
    *issued = true;
    return NUDIM_OK;
}

// The serving loop's step: queue the job's next iteration unless it waits on
// a residual check whose result has not arrived (never blocks the host).
int job_try_step(nudim_job *jb, bool *issued)
{
    *issued = false;
    if (!jb || !jb->ready) {
        set_error("job_try_step: job not ready");
        return NUDIM_ESTATE;
    }
    NUDIM_CUDA(cudaSetDevice(jb->ctx->device));
    return job_advance(jb, false, issued);
}

static int validate(const nudim_job_desc *d)
{
    if (!d) {
        set_error("null descriptor");
        return NUDIM_EINVAL;
    }
    if (d->nx <= 0 || d->nz <= 0 || d->np <= 0) {
        set_error("You need to provide valid projection size with --nx, --nz, --pad.");
        return NUDIM_EINVAL;
    }
    if ((d->nz & 1) || (d->np & 1)) {
        set_error("np and nz must be even (got np=%d nz=%d)", d->np, d->nz);
        return NUDIM_EINVAL;
    }
    if (d->nx > d->np) {
        set_error("nx (%d) must not exceed np (%d)", d->nx, d->np);
        return NUDIM_EINVAL;
    }
    if (d->nhio < 0 || d->ner < 0) {
        set_error("You need to provide valid nhio/ner.");
        return NUDIM_EINVAL;
    }
    if (!(d->interval > 0)) {
        set_error("You need to provide valid angular sampling interval with --interval.");
        return NUDIM_EINVAL;
    }
    if (!(d->padangle > 0) ||
        d->interval / d->padangle - (int)(d->interval / d->padangle + 0.1) > 1e-5) {
        set_error("You need to provide valid padded angular sampling interval with --padangle.");
        return NUDIM_EINVAL;
    }
    if (d->gam_max < -90 || d->gam_max > 90 || d->gam_min < -90 || d->gam_min > d->gam_max) {
        set_error("You need to provide valid scope of tomogram angles (-90,90] with --max, --min.");
        return NUDIM_EINVAL;
    }
    if (d->height && (d->nheight <= 0 || (d->variant == NUDIM_VARIANT_SERIAL && d->ncenter <= 0))) {
        set_error("You must provide valid both sample height and center with --height and --center.");
        return NUDIM_EINVAL;
    }
    if (d->denoise < 0 || d->denoise > 2 || d->precision < 0 || d->precision > 1 ||
        d->variant < 0 || d->variant > 1) {
        set_error("invalid enum value in descriptor");
        return NUDIM_EINVAL;
    }
    return NUDIM_OK;
}

// scratch of one fused NFFT pass (a chunk of planes: row spectra + partials
// in the trafo, column spectra + the oversampled grid in the adjoint):
// NUDIM_FUSED_BUDGET_MB, default 3 GB (all Z-planes of most jobs in one pass)
static size_t fused_budget_default()
{
    const char *fb = getenv("NUDIM_FUSED_BUDGET_MB");
    return fb ? (size_t)atol(fb) << 20 : ((size_t)3072 << 20);
}

static size_t job_bytes(const nudim_job_desc *d, int A, bool both, size_t fused_budget)
{
    size_t nz = d->nz, np = d->np, P2 = np * np, V = P2 * nz, M = (size_t)A * np;
    size_t n1 = (size_t)grid_size(d->np);
    auto per = [&](size_t sT) {
        size_t sC = 2 * sT;
        size_t b = 3 * V * sT + 3 * V * sC + 4 * nz * M * sC;  // + the initial volume
        if (d->denoise == NUDIM_DENOISE_TV) b += V * sT;
        b += M * (8 + 28 * sT + 20);  // node tables and tile lists
        // fused-path lists: ~11 adjoint tile entries and <= 5 trafo entries per
        // node (4-column blocks): id + 12 weights, and 3 ints + 20 weights
        b += M * (11 * (4 + 12 * sT) + 5 * (12 + 20 * sT));
        b += nz * (size_t)cgnr_part_stride((int)M, (int)P2) * 8;
        // fused-path workspace: row spectra + partials (trafo) or column
        // spectra + grid (adjoint) of one chunk of planes
        size_t plane = (np * n1 + std::max(5 * M, n1 * n1)) * sC, chunk = fused_budget / plane;
        b += (chunk < 1 ? 1 : chunk < nz ? chunk : nz) * plane;
        // FP32 CGNR by Toeplitz embedding (grids of 256 to 1024 points): T p
        // and the kernel's DFT
        if (sT == 4 && n1 >= 256 && n1 <= 1024) b += V * sC + n1 * n1 * sC;
        return b;
    };
    size_t b = d->precision == NUDIM_FP64 ? per(8) : per(4);
    if (both) b += per(8);
    return b;
}

}  // namespace nudim

// ================================================================ C ABI
extern "C" {

const char *nudim_last_error(void) { return nudim::last_error(); }
int nudim_abi_version(void) { return NUDIM_ABI_VERSION; }

int nudim_ctx_create(int device, unsigned flags, nudim_ctx **out)
{
    if (!out) {
        set_error("null output pointer");
        return NUDIM_EINVAL;
    }
    *out = nullptr;
    int n = 0;
    NUDIM_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) {
        set_error("device %d out of range (%d devices)", device, n);
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(device));
    auto *c = new nudim_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    const char *gb = getenv("NUDIM_GRID_BUDGET_MB");
    c->grid_budget = gb ? (size_t)atol(gb) << 20 : ((size_t)2 << 30);
    c->fused_budget = fused_budget_default();
    c->use_fused = !(flags & NUDIM_CTX_GRID_NFFT);
    c->autotune = (flags & NUDIM_CTX_AUTOTUNE) != 0;
    *out = c;
    return NUDIM_OK;
}

int nudim_ctx_destroy(nudim_ctx *c)
{
    if (!c) return NUDIM_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto &kv : c->fft2d) cufftDestroy(kv.second);
    for (auto &kv : c->fftz) cufftDestroy(kv.second);
    cudaFree(c->ws);
    cudaFree(c->scratch);
    cudaStreamDestroy(c->stream);
    delete c;
    return NUDIM_OK;
}

void *nudim_ctx_stream(nudim_ctx *c) { return c ? (void *)c->stream : nullptr; }

int nudim_ctx_profile(nudim_ctx *c, int enable)
{
    if (!c) return NUDIM_EINVAL;
    NUDIM_CUDA(cudaSetDevice(c->device));
    prof_collect(c);
    for (int k = 0; k < PK_COUNT; k++) {
        c->prof_ms[k] = 0;
        c->prof_n[k] = 0;
        c->prof_bytes[k] = 0;
    }
    c->prof_on = enable != 0;
    return NUDIM_OK;
}

int nudim_ctx_profile_read(nudim_ctx *c, int k, double *total_ms, long long *launches,
                           double *bytes)
{
    if (!c || k < 0 || k >= PK_COUNT) return NUDIM_EINVAL;
    NUDIM_CUDA(cudaSetDevice(c->device));
    prof_collect(c);
    if (total_ms) *total_ms = c->prof_ms[k];
    if (launches) *launches = c->prof_n[k];
    if (bytes) *bytes = c->prof_bytes[k];
    return NUDIM_OK;
}

int nudim_profile_kernel_count(void) { return PK_COUNT; }

const char *nudim_profile_kernel_name(int k)
{
    static const char *names[PK_COUNT] = {"pad",   "fft2d",  "interp", "spread",    "crop",
                                          "cgvec", "zfft",   "volume", "tv",        "diffusion",
                                          "toeplitz"};
    return (k >= 0 && k < PK_COUNT) ? names[k] : nullptr;
}

unsigned long long nudim_launch_count(void) { return g_launches; }

int nudim_ctx_sync(nudim_ctx *c)
{
    if (!c) return NUDIM_EINVAL;
    NUDIM_CUDA(cudaSetDevice(c->device));
    // jobs run on their own streams: wait for all work on the device
    NUDIM_CUDA(cudaDeviceSynchronize());
    return NUDIM_OK;
}

void *nudim_job_stream(nudim_job *jb) { return jb ? (void *)jb->stream : nullptr; }

int nudim_job_sync(nudim_job *jb)
{
    if (!jb) return NUDIM_EINVAL;
    NUDIM_CUDA(cudaSetDevice(jb->ctx->device));
    NUDIM_CUDA(cudaStreamSynchronize(jb->stream));
    return NUDIM_OK;
}

int nudim_job_footprint(const nudim_job_desc *d, size_t *bytes)
{
    NUDIM_TRY(validate(d));
    int A = polar_lines(d->gam_min, d->interval, d->padangle, nullptr, nullptr);
    *bytes = job_bytes(d, A, d->precision == NUDIM_MIXED && d->correct_every != 0,
                       fused_budget_default());
    return NUDIM_OK;
}

int nudim_job_create(nudim_ctx *ctx, const nudim_job_desc *desc, nudim_job **out)
{
    if (!ctx || !out) {
        set_error("null argument");
        return NUDIM_EINVAL;
    }
    *out = nullptr;
    NUDIM_TRY(validate(desc));
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    std::unique_ptr<nudim_job> jb(new nudim_job());
    jb->ctx = ctx;
    NUDIM_CUDA(cudaStreamCreateWithFlags(&jb->stream, cudaStreamNonBlocking));
    jb->ws.st = jb->stream;
    // on any early return below, release what was created so far
    struct Guard {
        nudim_job *j;
        ~Guard()
        {
            if (!j) return;
            j->s64.release();
            j->s32.release();
            ws_release(&j->ws);
            cudaStreamSynchronize(j->stream);
            cudaStreamDestroy(j->stream);
            if (j->check_ev) cudaEventDestroy(j->check_ev);
            if (j->check_host) cudaFreeHost(j->check_host);
        }
    } guard{jb.get()};
    jb->d = *desc;
    nudim_job_desc &d = jb->d;
    jb->nmeas = (int)((d.gam_max - d.gam_min) / d.interval + 0.5) + 1;
    jb->A = polar_lines(d.gam_min, d.interval, d.padangle, &jb->pad_min, &jb->pad_max);
    jb->M = jb->A * d.np;
    std::vector<double> x((size_t)jb->M * 2);
    equal_angle_sample_2d(jb->pad_min, jb->pad_max, d.padangle, d.np, x.data());
    if (build_nfft_tables(d.np, d.np, jb->M, x.data(), 16, 16, &jb->tabs) != 0) {
        set_error("invalid NFFT geometry");
        return NUDIM_EINVAL;
    }
    classify_lines(jb->pad_min, d.padangle, d.gam_min, d.gam_max, d.interval, jb->A, &jb->known,
                   &jb->order);
    for (int a = 0; a < jb->A; a++)
        if (jb->known[a] && jb->order[a] >= jb->nmeas) {
            set_error("tilt index out of range");
            return NUDIM_EINVAL;
        }
    jb->unk_rank.assign(jb->M, 0);
    int cnt = 0;
    for (int i = 0; i < jb->M; i++) {
        jb->unk_rank[i] = cnt;
        if (!jb->known[i / d.np]) cnt++;
    }
    jb->n_unk_row = cnt;
    if (d.precision == NUDIM_FP64) {
        NUDIM_TRY(state_init<double>(jb.get(), jb->s64));
    } else {
        NUDIM_TRY(state_init<float>(jb.get(), jb->s32));
        if (d.correct_every != 0) {
            NUDIM_TRY(state_init<double>(jb.get(), jb->s64));
            NUDIM_CUDA(cudaMallocHost(&jb->check_host, 2 * sizeof(double)));
            NUDIM_CUDA(cudaEventCreateWithFlags(&jb->check_ev, cudaEventDisableTiming));
        }
    }
    guard.j = nullptr;
    *out = jb.release();
    return NUDIM_OK;
}

int nudim_job_destroy(nudim_job *jb)
{
    if (!jb) return NUDIM_OK;
    cudaSetDevice(jb->ctx->device);
    jb->s64.release();
    jb->s32.release();
    ws_release(&jb->ws);
    if (jb->vol0) cudaFreeAsync(jb->vol0, jb->stream);
    cudaStreamSynchronize(jb->stream);
    cudaStreamDestroy(jb->stream);
    if (jb->check_ev) cudaEventDestroy(jb->check_ev);
    if (jb->check_host) cudaFreeHost(jb->check_host);
    delete jb;
    return NUDIM_OK;
}

int nudim_job_import_fill(nudim_job *jb, const double *fill, size_t n)
{
    if (!jb || (!fill && n)) return NUDIM_EINVAL;
    size_t need = (size_t)jb->n_unk_row * jb->d.nz;
    if (n != need) {
        set_error("fill has %zu values, the job has %zu unknown samples", n, need);
        return NUDIM_EINVAL;
    }
    jb->fill.assign(fill, fill + n);
    jb->fill_set = true;
    return NUDIM_OK;
}

int nudim_job_set_projections(nudim_job *jb, const double *proj, size_t n)
{
    if (!jb || !proj) {
        set_error("null argument");
        return NUDIM_EINVAL;
    }
    const nudim_job_desc &d = jb->d;
    size_t need = (size_t)jb->nmeas * d.nz * d.nx;
    if (n != need) {
        set_error("projections: got %zu values, need %d tilts x %d x %d = %zu", n, jb->nmeas, d.nz,
                  d.nx, need);
        return NUDIM_EINVAL;
    }
    nudim_ctx *ctx = jb->ctx;
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = jb->stream;
    // ---- tilt-series NFFT (reconstruction.c:307-367), FP64
    int M1 = d.np * d.nz;
    std::vector<double> x1((size_t)M1 * 2);
    uniform_sample_2d(d.np, d.nz, x1.data());
    NfftTables t1;
    if (build_nfft_tables(d.nx, d.nz, M1, x1.data(), 16, 16, &t1) != 0) {
        set_error("invalid tilt-series geometry (nx and nz must be even)");
        return NUDIM_EINVAL;
    }
    NfftDev<double> p1;
    p1.trafo_only = true;  // one trafo of the tilt series: no adjoint lists
    int rc = p1.init(ctx, t1, st, &jb->ws);
    std::vector<void *> tmp;
    auto talloc = [&](size_t b) -> void * {
        void *q = nullptr;
        if (cudaMallocAsync(&q, b, st) != cudaSuccess) return nullptr;
        tmp.push_back(q);
        return q;
    };
    auto cleanup = [&]() {
        for (void *q : tmp) cudaFreeAsync(q, st);
        p1.release();
        ws_release(&jb->ws);  // the tilt-series NFFT's scratch
        cudaStreamSynchronize(st);
    };
    double *d_proj = nullptr;
    double2 *d_fh = nullptr, *d_tomo = nullptr;
    int *d_order = nullptr, *d_rank = nullptr;
    double *d_fill = nullptr;
    if (!rc) {
        d_proj = (double *)talloc(sizeof(double) * n);
        d_fh = (double2 *)talloc(sizeof(double2) * n);
        d_tomo = (double2 *)talloc(sizeof(double2) * (size_t)jb->nmeas * M1);
        d_order = (int *)talloc(sizeof(int) * jb->A);
        d_rank = (int *)talloc(sizeof(int) * jb->M);
        if (!d_proj || !d_fh || !d_tomo || !d_order || !d_rank) {
            set_error("out of device memory for the tilt series");
            rc = NUDIM_ENOMEM;
        }
    }
    if (!rc && d.random) {
        size_t nf = (size_t)jb->n_unk_row * d.nz;
        if (!jb->fill_set) {
            jb->fill.resize(nf);
            mt19937_uniform(0, nf, jb->fill.data());
            for (double &v : jb->fill) v *= 10;  // gsl_rng_uniform(rng)*10
        }
        d_fill = (double *)talloc(sizeof(double) * (nf ? nf : 1));
        if (!d_fill) rc = NUDIM_ENOMEM;
        else if (nf) rc = cudaMemcpyAsync(d_fill, jb->fill.data(), sizeof(double) * nf,
                                          cudaMemcpyHostToDevice, st) ? NUDIM_ECUDA : NUDIM_OK;
    }
    if (!rc) {
        cudaMemcpyAsync(d_proj, proj, sizeof(double) * n, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_order, jb->order.data(), sizeof(int) * jb->A, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_rank, jb->unk_rank.data(), sizeof(int) * jb->M, cudaMemcpyHostToDevice,
                        st);
        k_proj_fhat<<<dim3(ceil_div((long)d.nx * d.nz, 256), jb->nmeas), 256, 0, st>>>(
            d_proj, d_fh, d.nx, d.nz);
        PadArgs<double> pa;
        pa.src = d_fh;
        pa.src_stride = (size_t)d.nx * d.nz;
        InterpArgs<double> ia;
        ia.out = d_tomo;
        ia.out_stride = M1;
        rc = p1.trafo(jb->nmeas, pa, ia, st);
    }
    // ---- reorder/mask/fill + initial inverse NFFT
    if (!rc) {
        jb->fp64_owns = false;
        if (d.precision == NUDIM_FP64)
            rc = state_setup<double>(jb, jb->s64, d_tomo, d_order, d_rank, d_fill);
        else {
            // a job whose HIO iterations run in FP64 starts from the FP64
            // initial inverse, so those iterations are the FP64 form's own
            const bool hio64 = d.correct_every < 0 && d.nhio > 0;
            rc = state_setup<float>(jb, jb->s32, d_tomo, d_order, d_rank, d_fill, !hio64);
            if (!rc && jb->s64.live)
                rc = state_setup<double>(jb, jb->s64, d_tomo, d_order, d_rank, d_fill, hio64);
            jb->fp64_owns = hio64;
        }
    }
    if (!rc) {
        // keep the initial volume: a device copy of the state's volume
        size_t V = (size_t)d.np * d.np * d.nz;
        size_t bytes = V * (d.precision == NUDIM_FP64 ? sizeof(double) : sizeof(float));
        const void *src = d.precision == NUDIM_FP64 ? (const void *)jb->s64.img_a
                                                    : (const void *)jb->s32.img_a;
        if (!jb->vol0 && cudaMallocAsync(&jb->vol0, bytes, st) != cudaSuccess) {
            jb->vol0 = nullptr;
            set_error("out of device memory for the initial volume");
            rc = NUDIM_ENOMEM;
        }
        if (!rc && jb->fp64_owns) {
            rc = launch_real_to<float>(jb->s64.img_a, (float *)jb->vol0, V, st);
        } else if (!rc && cudaMemcpyAsync(jb->vol0, src, bytes, cudaMemcpyDeviceToDevice, st) !=
                              cudaSuccess) {
            set_error("initial volume copy failed");
            rc = NUDIM_ECUDA;
        }
    }
    cleanup();
    if (!rc) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "set_projections", __FILE__, __LINE__);
        jb->ready = true;
        jb->done = 0;
    }
    return rc;
}

int nudim_step(nudim_ctx *ctx, nudim_job *const *jobs, int njobs, int iters)
{
    if (!ctx || (!jobs && njobs) || iters < 0) {
        set_error("invalid nudim_step arguments");
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    std::vector<int> target(njobs);
    for (int k = 0; k < njobs; k++) {
        nudim_job *jb = jobs[k];
        if (!jb || jb->ctx != ctx) {
            set_error("job %d does not belong to this context", k);
            return NUDIM_EINVAL;
        }
        if (!jb->ready) {
            set_error("nudim_step before nudim_job_set_projections");
            return NUDIM_ESTATE;
        }
        target[k] = std::min(jb->done + iters, jb->d.nhio + jb->d.ner);
    }
    // Round-robin: one iteration of each job per round.  A job whose next
    // iteration waits on its residual check's result is passed over until
    // the result is in; the host blocks only when every remaining iteration
    // waits on one.
    for (;;) {
        bool left = false, progress = false;
        for (int k = 0; k < njobs; k++) {
            if (jobs[k]->done >= target[k]) continue;
            left = true;
            bool issued = false;
            NUDIM_TRY(job_advance(jobs[k], false, &issued));
            progress = progress || issued;
        }
        if (!left) break;
        if (!progress)
            for (int k = 0; k < njobs; k++)
                if (jobs[k]->done < target[k]) {
                    bool issued = false;
                    NUDIM_TRY(job_advance(jobs[k], true, &issued));
                    break;
                }
    }
    return NUDIM_OK;
}

int nudim_job_get_volume(nudim_job *jb, double *out, size_t n, int crop)
{
    if (!jb || !out) return NUDIM_EINVAL;
    const nudim_job_desc &d = jb->d;
    size_t P2 = (size_t)d.np * d.np, V = P2 * d.nz;
    size_t need = crop ? (size_t)d.nz * d.nx * d.nx : V;
    if (n != need) {
        set_error("volume buffer has %zu values, need %zu", n, need);
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(jb->ctx->device));
    cudaStream_t st = jb->stream;
    std::vector<double> full;
    double *dst = crop ? (full.resize(V), full.data()) : out;
    if (d.precision == NUDIM_FP64 || jb->fp64_owns) {
        NUDIM_CUDA(cudaMemcpyAsync(dst, jb->s64.img_a, sizeof(double) * V, cudaMemcpyDeviceToHost, st));
    } else {
        double *tmpd = (double *)jb->s32.z;  // V complex floats = V doubles of room
        NUDIM_TRY(launch_to_double<float>(jb->s32.img_a, tmpd, V, st));
        NUDIM_CUDA(cudaMemcpyAsync(dst, tmpd, sizeof(double) * V, cudaMemcpyDeviceToHost, st));
    }
    NUDIM_CUDA(cudaStreamSynchronize(st));
    if (crop) {
        int lo = (d.np - d.nx) / 2, hi = (d.np + d.nx) / 2;
        size_t q = 0;
        for (int i = 0; i < d.nz; i++)
            for (int j = lo; j < hi; j++)
                for (int k = lo; k < hi; k++) out[q++] = full[((size_t)i * d.np + j) * d.np + k];
    }
    return NUDIM_OK;
}

int nudim_job_get_initial_volume(nudim_job *jb, double *out, size_t n)
{
    if (!jb || !out) return NUDIM_EINVAL;
    const nudim_job_desc &d = jb->d;
    size_t V = (size_t)d.np * d.np * d.nz;
    if (!jb->ready || !jb->vol0 || n != V) {
        set_error("initial volume unavailable or wrong size");
        return jb->ready ? NUDIM_EINVAL : NUDIM_ESTATE;
    }
    NUDIM_CUDA(cudaSetDevice(jb->ctx->device));
    cudaStream_t st = jb->stream;
    if (d.precision == NUDIM_FP64) {
        NUDIM_CUDA(cudaMemcpyAsync(out, jb->vol0, sizeof(double) * V, cudaMemcpyDeviceToHost, st));
    } else {
        // widened in the state's CGNR scratch (V complex floats = V doubles of
        // room), in stream order with the job's iterations
        double *tmpd = (double *)jb->s32.z;
        NUDIM_TRY(launch_to_double<float>((const float *)jb->vol0, tmpd, V, st));
        NUDIM_CUDA(cudaMemcpyAsync(out, tmpd, sizeof(double) * V, cudaMemcpyDeviceToHost, st));
    }
    NUDIM_CUDA(cudaStreamSynchronize(st));
    return NUDIM_OK;
}

int nudim_job_get_rfactor(nudim_job *jb, double *hist, int cap, int *count)
{
    if (!jb || (!hist && cap > 0)) return NUDIM_EINVAL;
    int n = std::min(cap, jb->done);
    if (n > 0) {
        NUDIM_CUDA(cudaSetDevice(jb->ctx->device));
        NUDIM_CUDA(cudaStreamSynchronize(jb->stream));
        double *src = jb->d.precision == NUDIM_FP64 ? jb->s64.rh : jb->s32.rh;
        NUDIM_CUDA(cudaMemcpy(hist, src, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    if (count) *count = n;
    return NUDIM_OK;
}

int nudim_job_iterations_done(nudim_job *jb, int *done)
{
    if (!jb || !done) return NUDIM_EINVAL;
    *done = jb->done;
    return NUDIM_OK;
}

int nudim_job_corrections(nudim_job *jb, int *count)
{
    if (!jb || !count) return NUDIM_EINVAL;
    *count = jb->corrections;
    return NUDIM_OK;
}

int nudim_job_set_denoise_dump(nudim_job *jb, int nn, double *before, double *after)
{
    if (!jb) return NUDIM_EINVAL;
    if (nn >= 0 && (!before || !after)) return NUDIM_EINVAL;
    jb->dump_nn = nn;
    jb->dump_before = before;
    jb->dump_after = after;
    return NUDIM_OK;
}

// ---------------------------------------------------------------- simulator
// method 0: -m 2D1D (Z-FFT + per-plane 2D NFFT); 1: -m DFT (exact sums with
// the reference's PI).  Both continue with the same 2D inverse FFT, shifts,
// noise and scaling.
static int project_run(nudim_ctx *ctx, int method, const double *density, int nx, int ny, int nz,
                       int np, double gam_min, double gam_max, double interval, double snr,
                       unsigned long seed, double *proj_out, size_t n_out)
{
    if (!ctx || !density || !proj_out || nx <= 0 || ny <= 0 || nz <= 0 || np <= 0 ||
        (nx | ny | nz | np) & 1 || !(interval > 0) || gam_min > gam_max || gam_min < -90 ||
        gam_max > 90) {
        set_error("invalid projection_sim arguments (sizes must be positive and even)");
        return NUDIM_EINVAL;
    }
    int ns = equal_angle_count(gam_min, gam_max, interval);
    if (n_out != (size_t)ns * nz * np) {
        set_error("output has %zu values, need %d tilts x %d x %d", n_out, ns, nz, np);
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    int M = ns * np;
    size_t XY = (size_t)nx * ny, V = XY * nz;
    std::vector<double> x((size_t)M * 2);
    equal_angle_sample_2d(gam_min, gam_max, interval, np, x.data());
    NfftDev<double> pl;
    int rc = NUDIM_OK;
    if (method == 0) {
        NfftTables t;
        build_nfft_tables(ny, nx, M, x.data(), 16, 16, &t);
        rc = pl.init(ctx, t);
    }
    double *dd = nullptr, *dout = nullptr;  // density (V) and tilt series (ns*nz*np)
    double2 *data = nullptr, *tmp = nullptr, *sl = nullptr;
    if (!rc && (cudaMalloc(&dd, sizeof(double) * V) ||
                (method == 0 && cudaMalloc(&data, sizeof(double2) * V)) ||
                cudaMalloc(&tmp, sizeof(double2) * (size_t)nz * M) ||
                cudaMalloc(&sl, sizeof(double2) * (size_t)ns * nz * np) ||
                cudaMalloc(&dout, sizeof(double) * (size_t)ns * nz * np))) {
        set_error("out of device memory in projection_sim");
        rc = NUDIM_ENOMEM;
    }
    cufftHandle hz = 0, h2 = 0;
    if (!rc) cudaMemcpyAsync(dd, density, sizeof(double) * V, cudaMemcpyHostToDevice, st);
    if (!rc && method == 1) {
        // :516-560: the exact sums; row j of tmp = the nodes of Z index j
        rc = dft_slices(dd, nx, ny, nz, np, x.data(), ns, tmp, (size_t)2 << 30, st);
    }
    if (!rc && method == 0) {
        k_real_cplx<<<ceil_div((long)V, 256), 256, 0, st>>>(dd, data, V);
        int n1[1] = {nz};
        // projection_sim.c:319-322: forward Z-FFT, stride nx*ny, unshifted
        if (cufftPlanMany(&hz, 1, n1, n1, (int)XY, 1, n1, (int)XY, 1, CUFFT_Z2Z, (int)XY) ||
            cufftSetStream(hz, st) ||
            cufftExecZ2Z(hz, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data,
                         CUFFT_FORWARD)) {
            set_error("cuFFT failure in projection_sim Z-FFT");
            rc = NUDIM_ECUDA;
        }
    }
    if (!rc && method == 0) {
        // :325-351 per plane NFFT; plane q of `data` is slice (q + nz/2) % nz
        PadArgs<double> pa;
        pa.src = data;
        pa.src_stride = XY;
        InterpArgs<double> ia;
        ia.out = tmp;
        ia.out_stride = M;
        rc = pl.trafo(nz, pa, ia, st);
    }
    if (!rc) {
        // :359-374 ifftshift into slice[row][col], 2D backward FFT per tilt
        const int zshift = method == 0 ? 0 : nz / 2;
        k_sim_gather<<<dim3(ceil_div((long)nz * np, 256), ns), 256, 0, st>>>(tmp, sl, nz, np, M,
                                                                             zshift);
        int n2[2] = {nz, np};
        if (cufftPlanMany(&h2, 2, n2, nullptr, 1, nz * np, nullptr, 1, nz * np, CUFFT_Z2Z, ns) ||
            cufftSetStream(h2, st) ||
            cufftExecZ2Z(h2, (cufftDoubleComplex *)sl, (cufftDoubleComplex *)sl, CUFFT_INVERSE)) {
            set_error("cuFFT failure in projection_sim 2D IFFT");
            rc = NUDIM_ECUDA;
        }
    }
    std::vector<double> host;
    if (!rc) {
        // :377-390 radial fftshift, keep the real part (scaled below)
        k_sim_shift<<<dim3(ceil_div((long)nz * np, 256), ns), 256, 0, st>>>(
            sl, dout, nz, np, method == 0 ? 0 : nz / 2);
        host.resize((size_t)ns * nz * np);
        cudaMemcpyAsync(host.data(), dout, sizeof(double) * host.size(), cudaMemcpyDeviceToHost,
                        st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "projection_sim", __FILE__, __LINE__);
    }
    if (!rc) {
        size_t per = (size_t)np * nz;
        std::vector<double> u;
        if (snr > 0) {
            u.resize(2 * per * ns);
            mt19937_uniform((uint32_t)seed, u.size(), u.data());
        }
        for (int j = 0; j < ns; j++) {
            double *s = host.data() + (size_t)j * per;
            if (snr > 0) {
                // add_noise (projection_sim.c:45-67): sigma of Re(slice)
                double sum = 0, sum2 = 0;
                for (size_t i = 0; i < per; i++) {
                    sum += s[i];
                    sum2 += s[i] * s[i];
                }
                double sigma = sqrt(sum2 / per - (sum / per) * (sum / per)) / snr;
                for (size_t i = 0; i < per; i++) {
                    // Box-Muller on consecutive uniforms of the seeded stream
                    size_t k = ((size_t)j * per + i);
                    double u1 = u[2 * k], u2 = u[2 * k + 1];
                    if (u1 <= 0) u1 = 1e-300;
                    s[i] += sigma * sqrt(-2.0 * log(u1)) * cos(2.0 * kTruePi * u2);
                }
            }
            for (size_t i = 0; i < per; i++) proj_out[(size_t)j * per + i] = s[i] / (np * nz);
        }
    }
    if (hz) cufftDestroy(hz);
    if (h2) cufftDestroy(h2);
    cudaStreamSynchronize(st);
    cudaFree(dd);
    cudaFree(dout);
    cudaFree(data);
    cudaFree(tmp);
    cudaFree(sl);
    pl.release();
    return rc;
}

int nudim_project_2d1d(nudim_ctx *ctx, const double *density, int nx, int ny, int nz, int np,
                       double gam_min, double gam_max, double interval, double snr,
                       unsigned long seed, double *proj_out, size_t n_out)
{
    return project_run(ctx, 0, density, nx, ny, nz, np, gam_min, gam_max, interval, snr, seed,
                       proj_out, n_out);
}

int nudim_project_dft(nudim_ctx *ctx, const double *density, int nx, int ny, int nz, int np,
                      double gam_min, double gam_max, double interval, double snr,
                      unsigned long seed, double *proj_out, size_t n_out)
{
    return project_run(ctx, 1, density, nx, ny, nz, np, gam_min, gam_max, interval, snr, seed,
                       proj_out, n_out);
}

// ---------------------------------------------------------------- operators
int nudim_nfft_plan_create(nudim_ctx *ctx, int N0, int N1, int M, const double *x,
                           int precision, nudim_nfft_plan **out)
{
    if (!ctx || !out || (!x && M) || M < 0 || (precision != 0 && precision != 1)) {
        set_error("invalid plan arguments");
        return NUDIM_EINVAL;
    }
    *out = nullptr;
    for (long j = 0; j < 2L * M; j++)
        if (!(x[j] >= -0.5 && x[j] < 0.5)) {
            set_error("node coordinate %ld out of [-1/2, 1/2)", j);
            return NUDIM_EINVAL;
        }
    NfftTables t;
    if (build_nfft_tables(N0, N1, M, x, 16, 16, &t) != 0) {
        set_error("N0 and N1 must be positive and even");
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    auto *p = new nudim_nfft_plan();
    p->ctx = ctx;
    p->prec = precision;
    int rc = precision == NUDIM_FP64 ? p->d64.init(ctx, t) : p->d32.init(ctx, t);
    // tables were uploaded on the legacy stream; callers may use any stream
    if (!rc) rc = cudaStreamSynchronize(nullptr) == cudaSuccess ? NUDIM_OK : NUDIM_ECUDA;
    if (rc) {
        p->d64.release();
        p->d32.release();
        delete p;
        return rc;
    }
    *out = p;
    return NUDIM_OK;
}

int nudim_nfft_plan_destroy(nudim_nfft_plan *p)
{
    if (!p) return NUDIM_OK;
    cudaSetDevice(p->ctx->device);
    cudaDeviceSynchronize();
    p->d64.release();
    p->d32.release();
    cudaFree(p->cg);
    delete p;
    return NUDIM_OK;
}

}  // extern "C"
template <typename T>
static int op_trafo(NfftDev<T> &d, int nplanes, const void *fh, void *f, cudaStream_t st)
{
    PadArgs<T> pa;
    pa.src = fh;
    pa.src_stride = (size_t)d.N0 * d.N1;
    InterpArgs<T> ia;
    ia.out = (cplx_t<T> *)f;
    ia.out_stride = d.M;
    return d.trafo(nplanes, pa, ia, st);
}

template <typename T>
static int op_adjoint(NfftDev<T> &d, int nplanes, const void *f, void *fh, cudaStream_t st)
{
    SpreadArgs<T> sa;
    sa.f = (const cplx_t<T> *)f;
    sa.f_stride = d.M;
    CropArgs<T> ca;
    ca.out = (cplx_t<T> *)fh;
    ca.out_stride = (size_t)d.N0 * d.N1;
    return d.adjoint(nplanes, sa, ca, st);
}

extern "C" {
int nudim_nfft_plan_tuning(nudim_nfft_plan *p, int *trafo_cols, int *spread_planes)
{
    if (!p || !trafo_cols || !spread_planes) return NUDIM_EINVAL;
    bool f = p->prec == NUDIM_FP64 ? p->d64.fused : p->d32.fused;
    *trafo_cols = !f ? 0 : p->prec == NUDIM_FP64 ? p->d64.BC : p->d32.BC;
    *spread_planes = !f ? 0 : p->prec == NUDIM_FP64 ? p->d64.Pa : p->d32.Pa;
    return NUDIM_OK;
}

int nudim_nfft_trafo(nudim_nfft_plan *p, int nplanes, const void *f_hat, void *f, void *stream)
{
    if (!p || nplanes < 0 || (nplanes && (!f_hat || !f))) return NUDIM_EINVAL;
    NUDIM_CUDA(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    return p->prec == NUDIM_FP64 ? op_trafo(p->d64, nplanes, f_hat, f, st)
                                 : op_trafo(p->d32, nplanes, f_hat, f, st);
}

int nudim_nfft_adjoint(nudim_nfft_plan *p, int nplanes, const void *f, void *f_hat, void *stream)
{
    if (!p || nplanes < 0 || (nplanes && (!f_hat || !f))) return NUDIM_EINVAL;
    NUDIM_CUDA(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    return p->prec == NUDIM_FP64 ? op_adjoint(p->d64, nplanes, f, f_hat, st)
                                 : op_adjoint(p->d32, nplanes, f, f_hat, st);
}

}  // extern "C"
template <typename T>
static int op_cgnr(nudim_nfft_plan *p, NfftDev<T> &d, int nplanes, const void *y, const void *w,
                   void *f, int iters, cudaStream_t st)
{
    using C = cplx_t<T>;
    size_t N = (size_t)d.N0 * d.N1, M = d.M;
    int stride = cgnr_part_stride((int)M, (int)N);
    size_t need = sizeof(C) * nplanes * (2 * M + 2 * N) +
                  sizeof(double) * ((size_t)nplanes * (stride + 4) + 8);
    if (need > p->cg_bytes) {
        cudaDeviceSynchronize();
        cudaFree(p->cg);
        p->cg = nullptr;
        p->cg_bytes = 0;
        NUDIM_CUDA(cudaMalloc(&p->cg, need));
        p->cg_bytes = need;
    }
    CgnrBuffers<T> b;
    char *base = (char *)p->cg;
    b.r = (C *)base;
    b.v = b.r + nplanes * M;
    b.z = b.v + nplanes * M;
    b.p = b.z + nplanes * N;
    b.part = (double *)(b.p + nplanes * N);
    b.part_stride = stride;
    b.dots = b.part + (size_t)nplanes * stride;
    return cgnr_run<T>(d, nplanes, (const C *)y, (const T *)w, (C *)f, nullptr, false, iters, b,
                       st);
}

extern "C" {
int nudim_cgnr(nudim_nfft_plan *p, int nplanes, const void *y, const void *w, void *f_hat_iter,
               int iters, void *stream)
{
    if (!p || nplanes < 0 || iters < 0 || (nplanes && (!y || !f_hat_iter))) return NUDIM_EINVAL;
    if (!nplanes) return NUDIM_OK;
    NUDIM_CUDA(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    return p->prec == NUDIM_FP64 ? op_cgnr(p, p->d64, nplanes, y, w, f_hat_iter, iters, st)
                                 : op_cgnr(p, p->d32, nplanes, y, w, f_hat_iter, iters, st);
}

int nudim_tv(nudim_ctx *ctx, int precision, void *vol, int nz, int ny, int nx, float lam,
             int niter, int height, int nheight, int ncenter, void *stream)
{
    if (!ctx || !vol || nz <= 0 || ny <= 0 || nx <= 0 || niter < 0 ||
        (precision != 0 && precision != 1)) {
        set_error("invalid nudim_tv arguments");
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    size_t V = (size_t)nz * ny * nx;
    int cap = tv_part_count(nz, ny, nx);
    size_t sT = precision == NUDIM_FP64 ? 8 : 4;
    double *scr;
    // partials and sums, then the gradient and the fused passes' second
    // volume and gradient (each 256-byte aligned)
    const size_t head = ((sizeof(double) * ((size_t)cap + 4)) + 255) & ~(size_t)255;
    const size_t vb = (sT * V + 255) & ~(size_t)255;
    NUDIM_TRY(ctx_scratch(ctx, head + 3 * vb, &scr));
    double *part = scr, *scal = scr + cap;
    unsigned char *grad = (unsigned char *)scr + head;
    int ylo = (2 * ncenter - nheight) / 2, yhi = (2 * ncenter + nheight) / 2;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == NUDIM_FP64)
        return tv_run<double>((double *)vol, (double *)grad, part, cap, scal, nz, ny, nx, lam,
                              niter, height ? 1 : 0, ylo, yhi, st, (double *)(grad + vb),
                              (double *)(grad + 2 * vb));
    return tv_run<float>((float *)vol, (float *)grad, part, cap, scal, nz, ny, nx, lam, niter,
                         height ? 1 : 0, ylo, yhi, st, (float *)(grad + vb),
                         (float *)(grad + 2 * vb));
}

int nudim_diffusion2d(nudim_ctx *ctx, int precision, void *vol, int nz, int ny, int nx,
                      int nx_bound, float lambda, float kappa, int niter, void *stream)
{
    if (!ctx || !vol || nz <= 0 || ny <= 0 || nx <= 0 || nx_bound <= 0 || niter < 0 ||
        (precision != 0 && precision != 1)) {
        set_error("invalid nudim_diffusion2d arguments");
        return NUDIM_EINVAL;
    }
    NUDIM_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == NUDIM_FP64)
        return diffusion_run<double>((double *)vol, nz, ny, nx, nx_bound, lambda, kappa, niter, st);
    return diffusion_run<float>((float *)vol, nz, ny, nx, nx_bound, lambda, kappa, niter, st);
}

}  // extern "C"
