// noalloc.cu -- total-variation denoising without any device allocation.
//
// Some callers cannot call cudaMalloc: a host program whose memory manager
// has already reserved the whole device (a pre-sized pool owned by another
// framework), or a latency-critical loop that must not hit the implicit
// device synchronisation cudaMalloc/cudaFree can cause.  For them
// nudim_tv_noalloc runs the same TV kernels as nudim_tv, but its scratch (the
// gradient field, the per-block partial sums and the two global sums) lives
// in the fixed file-scope device array below instead of context memory.
//
// The array is kNoAllocScratchBytes (32 MiB) and exists on every GPU that
// loads this library, for the life of the process.  Calls share it: two
// calls whose work overlaps on a GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the
// caller.  Every scratch element a call reads is written earlier in the same
// call, so nothing needs clearing between calls.
#include <mutex>

#include "engine.cuh"

namespace nudim {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch in the CUDA context current on the
// calling thread.  In host code the array's name is only a host-side handle,
// never a device address, so the address is looked up with
// cudaGetSymbolAddress, with that device and context current, the first
// time a context uses the array, and cached per device together with the
// context's process-unique ID (cuCtxGetId).  A call from another context on
// the same device -- after cudaDeviceReset, or from a driver-API or green
// context -- has another ID and looks the address up again, so a stale
// address is never handed to a kernel.  The two driver calls are reached
// through cudaGetDriverEntryPointByVersion, so the library does not link
// libcuda directly.
typedef int (*ctx_get_current_fn)(void **ctx);
typedef int (*ctx_get_id_fn)(void *ctx, unsigned long long *id);

struct NoAllocSlot {
    unsigned long long ctx_id = 0;
    bool set = false;
    void *addr = nullptr;
};

static std::mutex g_noalloc_mu;
static NoAllocSlot g_noalloc_slot[128];
static ctx_get_current_fn g_ctx_current = nullptr;
static ctx_get_id_fn g_ctx_id = nullptr;

static int driver_entry(const char *name, void **fn)
{
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return cuda_fail(e, name, __FILE__, __LINE__);
    if (q != cudaDriverEntryPointSuccess || !*fn) {
        set_error("nudim_tv_noalloc: driver entry point %s unavailable", name);
        return NUDIM_ECUDA;
    }
    return NUDIM_OK;
}

// The ID of the context current on this thread (0 when none is current yet).
static int current_ctx_id(unsigned long long *id)
{
    void *cu = nullptr;
    *id = 0;
    if (g_ctx_current(&cu) != 0) {
        set_error("nudim_tv_noalloc: cuCtxGetCurrent failed");
        return NUDIM_ECUDA;
    }
    if (cu && g_ctx_id(cu, id) != 0) {
        set_error("nudim_tv_noalloc: cuCtxGetId failed");
        return NUDIM_ECUDA;
    }
    return NUDIM_OK;
}

static int noalloc_scratch(int dev, void **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (dev < 0 || dev >= 128) {
        set_error("device index %d out of range", dev);
        return NUDIM_EINVAL;
    }
    if (!g_ctx_current) NUDIM_TRY(driver_entry("cuCtxGetCurrent", (void **)&g_ctx_current));
    if (!g_ctx_id) NUDIM_TRY(driver_entry("cuCtxGetId", (void **)&g_ctx_id));
    unsigned long long id = 0;
    NUDIM_TRY(current_ctx_id(&id));
    NoAllocSlot &s = g_noalloc_slot[dev];
    if (!s.set || id == 0 || s.ctx_id != id) {
        // set-up for this device and context (makes the runtime's primary
        // context current when no context was current yet)
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
        NUDIM_TRY(current_ctx_id(&id));
        s.addr = p;
        s.ctx_id = id;
        s.set = id != 0;
    }
    *out = s.addr;
    return NUDIM_OK;
}

}  // namespace nudim

using namespace nudim;

extern "C" int nudim_tv_noalloc(int precision, void *vol, int nz, int ny, int nx, float lam,
                                int niter, int height, int nheight, int ncenter, void *stream)
{
    if (!vol || nz <= 0 || ny <= 0 || nx <= 0 || niter < 0 ||
        (precision != NUDIM_FP64 && precision != NUDIM_MIXED)) {
        set_error("invalid nudim_tv_noalloc arguments");
        return NUDIM_EINVAL;
    }
    size_t V = (size_t)nz * ny * nx;
    size_t sT = precision == NUDIM_FP64 ? sizeof(double) : sizeof(float);
    int cap = tv_part_count(nz, ny, nx);
    size_t head = ((sizeof(double) * ((size_t)cap + 4)) + 255) & ~(size_t)255;
    size_t need = head + sT * V;
    if (need > kNoAllocScratchBytes) {
        set_error("nudim_tv_noalloc: a %d x %d x %d volume needs %zu bytes of scratch; the "
                  "fixed scratch holds %zu bytes (use nudim_tv for larger volumes)",
                  nz, ny, nx, need, kNoAllocScratchBytes);
        return NUDIM_EINVAL;
    }
    int dev = 0;
    NUDIM_CUDA(cudaGetDevice(&dev));
    void *base = nullptr;
    NUDIM_TRY(noalloc_scratch(dev, &base));
    double *part = (double *)base, *scal = part + cap;
    void *grad = (unsigned char *)base + head;
    int ylo = (2 * ncenter - nheight) / 2, yhi = (2 * ncenter + nheight) / 2;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == NUDIM_FP64)
        return tv_run<double>((double *)vol, (double *)grad, part, cap, scal, nz, ny, nx, lam,
                              niter, height ? 1 : 0, ylo, yhi, st);
    return tv_run<float>((float *)vol, (float *)grad, part, cap, scal, nz, ny, nx, lam, niter,
                         height ? 1 : 0, ylo, yhi, st);
}
