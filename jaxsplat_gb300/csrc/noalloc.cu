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

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned long long *g_scratch[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the calling thread's current device.
// In host code the array's name is only a stand-in for the symbol, never a
// device address, so the address is looked up once per device (with that
// device current) and cached.
int scratch_on_current_device(unsigned long long **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail(SPLAT_ERR_INVALID_ARG, "device ordinal %d outside [0, %d)", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(SPLAT_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s",
                        cudaGetErrorString(e));
        g_scratch[dev] = static_cast<unsigned long long *>(ptr);
    }
    *out = g_scratch[dev];
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
    if (int rc = scratch_on_current_device(&scratch)) return rc;
    int64_t *total = total_out ? total_out
                               : reinterpret_cast<int64_t *>(scratch + kNoAllocWords - 1);
    // launch_project_fwd zeroes the ticket and look-back words it uses
    // before the kernel reads them.
    return launch_project_fwd(*p, means3d, scales, quats, viewmat, cov3d, xys, depths, radii,
                              conics, compensation, num_tiles_hit, cum_tiles_hit, total, scratch,
                              nullptr, nullptr, nullptr, s);
}
