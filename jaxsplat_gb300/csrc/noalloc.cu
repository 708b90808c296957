// noalloc.cu -- projection forward for callers that cannot allocate.
//
// Some hosts hand this library their device buffers but no way to allocate
// more: a renderer plugin whose host application owns and pools all device
// memory, or a custom-call handler of another runtime that runs where a
// cudaMalloc would synchronise the device or is not permitted.  For them,
// splat_project_fwd_noalloc does the same work as splat_project_fwd without a
// workspace argument: the scan's look-back words live in the file-scope
// device array below, so nothing is allocated per call.
//
// Costs and rules of that choice:
//  * every GPU that loads the library holds the array (about 0.5 MB) until
//    the process exits;
//  * it bounds the problem size: at most kNoAllocMaxPoints Gaussians;
//  * all calls on a device share the one array, so calls that overlap on the
//    GPU (different streams, no ordering between them) race and corrupt each
//    other's scan; callers must order them;
//  * the array keeps the previous call's contents: each call clears the words
//    it uses before its kernel runs (a cudaMemsetAsync, not an allocation).
#include <mutex>

#include "splat_internal.cuh"

namespace splat {

int launch_project_fwd(const splat_params &, const float *, const float *, const float *,
                       const float *, float *, float *, float *, int32_t *, float *, float *,
                       int32_t *, int32_t *, int64_t *, unsigned long long *, const float *, const float *, float *,
                       cudaStream_t);
int check_params(const splat_params *p);

constexpr uint32_t kNoAllocMaxPoints = 1u << 24;
// word 0: partition ticket; words 1..P: one look-back word per partition of
// the projection (4096 Gaussians; the array allows one per 256, so it never
// runs short); last word: the 64-bit intersection total when the caller
// passes no total_out.
constexpr size_t kNoAllocWords = 1 + (kNoAllocMaxPoints + 255) / 256 + 1;

static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocWords];

namespace {

// A __device__ array has its own address in every CUDA context that loads
// the library: one per device's primary context, a new one after
// cudaDeviceReset recreates that context, and another in any context a host
// creates and makes current with the driver API.  The address is therefore
// cached per context, keyed by the context's ID (unique for the life of the
// process, never reused), not per device ordinal.  The driver calls come
// through cudaGetDriverEntryPointByVersion so that the library does not link
// libcuda (it still loads on machines without a driver).
typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);
typedef int (*StreamGetCtxFn)(void *stream, void **ctx);

struct DriverFns {
    CtxGetCurrentFn ctx_get_current = nullptr;
    CtxGetIdFn ctx_get_id = nullptr;
    StreamGetCtxFn stream_get_ctx = nullptr;
};

constexpr int kMaxContexts = 64;
struct CachedScratch {
    unsigned long long ctx_id;
    unsigned long long *ptr;
};
std::mutex g_mutex;
DriverFns g_fns;
bool g_fns_loaded = false;
CachedScratch g_cache[kMaxContexts];
int g_cache_len = 0;
int g_cache_next = 0;  // round-robin slot once the table is full

int load_driver_fns() {
    if (g_fns_loaded) return SPLAT_OK;
    struct {
        const char *name;
        void **slot;
    } want[] = {{"cuCtxGetCurrent", reinterpret_cast<void **>(&g_fns.ctx_get_current)},
                {"cuCtxGetId", reinterpret_cast<void **>(&g_fns.ctx_get_id)},
                {"cuStreamGetCtx", reinterpret_cast<void **>(&g_fns.stream_get_ctx)}};
    for (auto &w : want) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        const cudaError_t e =
            cudaGetDriverEntryPointByVersion(w.name, w.slot, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*w.slot)
            return fail(SPLAT_ERR_CUDA, "driver entry point %s unavailable (%s)", w.name,
                        cudaGetErrorString(e));
    }
    g_fns_loaded = true;
    return SPLAT_OK;
}

// Device address of g_noalloc_scratch in the calling thread's current
// context, and a check that `stream` belongs to that context.  In host code
// the array's name is only a stand-in for the symbol, never a device
// address, so the address is looked up with cudaGetSymbolAddress the first
// time a context is seen (with that context current) and cached.
int scratch_for_stream(cudaStream_t stream, unsigned long long **out) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (int rc = load_driver_fns()) return rc;
    void *ctx = nullptr;
    if (g_fns.ctx_get_current(&ctx) != 0)
        return fail(SPLAT_ERR_CUDA, "cuCtxGetCurrent failed");
    void *ptr = nullptr;
    if (!ctx) {
        // No context yet on this thread: the runtime call below makes the
        // current device's primary context current.
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(SPLAT_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s",
                        cudaGetErrorString(e));
        if (g_fns.ctx_get_current(&ctx) != 0 || !ctx)
            return fail(SPLAT_ERR_CUDA, "no current CUDA context");
    }
    void *stream_ctx = nullptr;
    if (g_fns.stream_get_ctx(reinterpret_cast<void *>(stream), &stream_ctx) != 0)
        return fail(SPLAT_ERR_INVALID_ARG, "cuStreamGetCtx failed for the given stream");
    if (stream_ctx != ctx)
        return fail(SPLAT_ERR_INVALID_ARG,
                    "the stream belongs to another CUDA context than the current one");
    unsigned long long id = 0;
    if (g_fns.ctx_get_id(ctx, &id) != 0) return fail(SPLAT_ERR_CUDA, "cuCtxGetId failed");
    for (int i = 0; i < g_cache_len; ++i) {
        if (g_cache[i].ctx_id == id) {
            *out = g_cache[i].ptr;
            return SPLAT_OK;
        }
    }
    if (!ptr) {
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(SPLAT_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s",
                        cudaGetErrorString(e));
    }
    const int slot = g_cache_len < kMaxContexts ? g_cache_len++ : (g_cache_next++ % kMaxContexts);
    g_cache[slot] = {id, static_cast<unsigned long long *>(ptr)};
    *out = g_cache[slot].ptr;
    return SPLAT_OK;
}

}  // namespace
}  // namespace splat

using namespace splat;

extern "C" int splat_project_fwd_noalloc(const splat_params *p, const float *means3d,
                                         const float *scales, const float *quats,
                                         const float *viewmat, float *cov3d, float *xys,
                                         float *depths, int32_t *radii, float *conics,
                                         float *compensation, int32_t *num_tiles_hit,
                                         int32_t *cum_tiles_hit, int64_t *total_out,
                                         splat_stream_t stream) {
    if (int rc = check_params(p)) return rc;
    if (p->num_points > kNoAllocMaxPoints)
        return fail(SPLAT_ERR_INVALID_ARG,
                    "splat_project_fwd_noalloc handles at most %u Gaussians (fixed scratch); "
                    "got %u: use splat_project_fwd with a workspace",
                    kNoAllocMaxPoints, p->num_points);
    cudaStream_t s = (cudaStream_t)stream;
    if (p->num_points == 0) {
        if (total_out && cudaMemsetAsync(total_out, 0, sizeof(int64_t), s) != cudaSuccess)
            return check_launch("total memset");
        return SPLAT_OK;
    }
    if (!means3d || !scales || !quats || !viewmat || !cov3d || !xys || !depths || !radii ||
        !conics || !compensation || !num_tiles_hit || !cum_tiles_hit)
        return fail(SPLAT_ERR_INVALID_ARG, "an input or output pointer is NULL");
    unsigned long long *scratch = nullptr;
    if (int rc = scratch_for_stream(s, &scratch)) return rc;
    int64_t *total = total_out ? total_out
                               : reinterpret_cast<int64_t *>(scratch + kNoAllocWords - 1);
    // launch_project_fwd zeroes the ticket and look-back words it uses
    // before the kernel reads them.
    return launch_project_fwd(*p, means3d, scales, quats, viewmat, cov3d, xys, depths, radii,
                              conics, compensation, num_tiles_hit, cum_tiles_hit, total, scratch,
                              nullptr, nullptr, nullptr, s);
}
