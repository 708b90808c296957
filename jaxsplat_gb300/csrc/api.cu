// api.cu -- the extern "C" entry points of libsplat (declared in include/splat.h).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "splat_internal.cuh"

namespace splat {

// kernels implemented in project.cu / sort.cu / raster.cu
int launch_project_fwd(const splat_params &, const float *, const float *, const float *,
                       const float *, float *, float *, float *, int32_t *, float *, float *,
                       int32_t *, int32_t *, int64_t *, unsigned long long *, const float *, const float *, float *,
                       cudaStream_t);
int launch_project_bwd(const splat_params &, const float *, const float *, const float *,
                       const float *, const float *, const int32_t *, const float *,
                       const float *, const float *, const float *, const float *,
                       const float *, float *, float *, float *, float *, float *, cudaStream_t);
size_t sort_workspace_bytes(const splat_params &, long long);
int launch_sort_and_bin(const splat_params &, Count, const float *, const float *,
                        const int32_t *, const int32_t *, int32_t *, int2 *, long long *,
                        int32_t *, long long *, void *, size_t, cudaStream_t);
int launch_pack(const splat_params &, const float *, const float *, const float *, const float *,
                float *, cudaStream_t);
int launch_raster_fwd(const splat_params &, Count, const int32_t *, const int2 *,
                      const float *, const float *, float *, int32_t *, float *, const float *,
                      float *, float *, uint8_t *, cudaStream_t);
int launch_raster_bwd(const splat_params &, Count, const int32_t *, const int2 *,
                      const float *, const float *, const float *, const int32_t *,
                      const float *, const float *, float *, float *, float *, float *, float *,
                      const uint8_t *, cudaStream_t);
int launch_count_pairs(const splat_params &, Count, const int32_t *, const int2 *, const float *,
                       const int32_t *, unsigned long long *, cudaStream_t);

static thread_local std::string g_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

int check_launch(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SPLAT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return SPLAT_OK;
}

// The largest tile grid handled: the scan carries per-block sums of 256 tile
// counts in 32 bits and the sort's look-back counts in 30 bits.
constexpr unsigned kMaxTiles = 1u << 22;
constexpr long long kMaxIntersects = (1ll << 30) - 1;

static int validate(const splat_params *p) {
    if (!p) return fail(SPLAT_ERR_INVALID_ARG, "params is NULL");
    if (p->block_width < 2 || p->block_width > 16)
        return fail(SPLAT_ERR_INVALID_ARG, "block_width must be in [2, 16], got %u", p->block_width);
    if (p->img_width == 0 || p->img_height == 0)
        return fail(SPLAT_ERR_INVALID_ARG, "image size must be positive, got %ux%u", p->img_height,
                    p->img_width);
    if ((unsigned long long)tiles_x(*p) * tiles_y(*p) > kMaxTiles)
        return fail(SPLAT_ERR_INVALID_ARG, "tile grid %ux%u exceeds %u tiles", tiles_x(*p),
                    tiles_y(*p), kMaxTiles);
    if (p->num_points > 0x7fffffffu)
        return fail(SPLAT_ERR_INVALID_ARG, "num_points %u exceeds int32", p->num_points);
    return SPLAT_OK;
}

// Parameter validation shared with the other translation units.
int check_params(const splat_params *p) { return validate(p); }

static int check_count(long long count) {
    if (count < 0 || count > kMaxIntersects)
        return fail(SPLAT_ERR_OVERFLOW, "intersection count %lld outside [0, %lld]", count,
                    kMaxIntersects);
    return SPLAT_OK;
}

#define NEED(ptr)                                                                          \
    do {                                                                                   \
        if (!(ptr)) return fail(SPLAT_ERR_INVALID_ARG, "%s is NULL", #ptr);               \
    } while (0)

// tile_bins is read and written as int2
#define NEED_BINS(ptr)                                                                     \
    do {                                                                                   \
        NEED(ptr);                                                                         \
        if (reinterpret_cast<uintptr_t>(ptr) % 8)                                          \
            return fail(SPLAT_ERR_INVALID_ARG, "%s must be 8-byte aligned", #ptr);         \
    } while (0)

// Workspaces hold 64-bit words updated by atomics and vector-loaded arrays:
// 256-byte aligned, as every device allocator returns them.
#define NEED_WS(ptr)                                                                       \
    do {                                                                                   \
        NEED(ptr);                                                                         \
        if (reinterpret_cast<uintptr_t>(ptr) % 256)                                        \
            return fail(SPLAT_ERR_INVALID_ARG, "%s must be 256-byte aligned", #ptr);       \
    } while (0)

static size_t project_ws_bytes(const splat_params &p) {
    // one look-back word per partition (4096 Gaussians; sized per 256)
    const size_t parts = (p.num_points + 255) / 256;
    return (parts + 2) * sizeof(unsigned long long) + 256;
}

// ---------------------------------------------------------------------------
// Device utilities.

__global__ void l2_loss_kernel(const float *img, const float *target, long long count,
                               float inv_count, float *loss, float *v_img) {
    float local = 0.f;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const float d = img[i] - target[i];
        v_img[i] = 2.f * d * inv_count;
        local += d * d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    __shared__ float s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) atomicAdd(loss, v * inv_count);
    }
}

__device__ unsigned long long g_never_set;  // zero for the life of the module

__global__ void wait_timeout_kernel(uint32_t limit, uint32_t *status) {
    if (threadIdx.x == 0) (void)wait_flagged(&g_never_set, limit, status);
}

// 80-byte descriptor with the layout of ops::Descriptor (lib/ops.h:9-22).
struct XlaDescriptor {
    uint32_t num_points;
    uint32_t img_shape[3];  // (W, H, 1)
    alignas(16) float intrins[4];
    float glob_scale;
    float clip_thresh;
    uint32_t block_width;
    uint32_t grid_dim_1d;
    uint32_t block_dim_1d;
    uint32_t grid_dim_2d[3];
    uint32_t block_dim_2d[3];
};
static_assert(sizeof(XlaDescriptor) == 80, "descriptor layout");

static int unpack(const char *opaque, size_t len, splat_params *p) {
    if (!opaque || len != sizeof(XlaDescriptor))
        return fail(SPLAT_ERR_INVALID_ARG, "Invalid opaque object size %zu (want %zu)", len,
                    sizeof(XlaDescriptor));
    XlaDescriptor d;
    std::memcpy(&d, opaque, sizeof(d));
    std::memset(p, 0, sizeof(*p));
    p->num_points = d.num_points;
    p->img_width = d.img_shape[0];
    p->img_height = d.img_shape[1];
    p->fx = d.intrins[0];
    p->fy = d.intrins[1];
    p->cx = d.intrins[2];
    p->cy = d.intrins[3];
    p->glob_scale = d.glob_scale;
    p->clip_thresh = d.clip_thresh;
    p->block_width = d.block_width;
    return validate(p);
}

static void report(const char *entry, int rc) {
    if (rc != SPLAT_OK) std::fprintf(stderr, "libsplat %s: %s\n", entry, g_error.c_str());
}

static int read_count(const int32_t *cum, uint32_t n, long long *out, cudaStream_t s) {
    int32_t v = 0;
    if (n > 0 && cudaMemcpyAsync(&v, cum + n - 1, sizeof(v), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return check_launch("intersection count read");
    if (cudaStreamSynchronize(s) != cudaSuccess) return check_launch("intersection count read");
    *out = v;
    return check_count(v);
}

}  // namespace splat

using namespace splat;

extern "C" {

const char *splat_last_error(void) { return g_error.c_str(); }

const char *splat_status_string(int status) {
    switch (status) {
    case SPLAT_OK: return "ok";
    case SPLAT_ERR_INVALID_ARG: return "invalid argument";
    case SPLAT_ERR_CUDA: return "CUDA error";
    case SPLAT_ERR_WORKSPACE: return "workspace too small";
    case SPLAT_ERR_OVERFLOW: return "intersection count out of range";
    case SPLAT_ERR_DEVICE: return "device-side check failed";
    default: return "unknown status";
    }
}

const char *splat_device_status_string(uint32_t bits) {
    static thread_local std::string s;
    s.clear();
    if (bits & DEV_LOOKBACK_TIMEOUT) s += "lookback-timeout ";
    if (bits & DEV_EMIT_OVERFLOW) s += "emit-overflow ";
    if (bits & DEV_SORT_OVERFLOW) s += "sort-overflow ";
    if (bits & DEV_SCAN_OVERFLOW) s += "scan-overflow ";
    if (bits & DEV_BAD_TILE) s += "bad-tile ";
    if (bits & DEV_BAD_ID) s += "bad-gaussian-id ";
    if (bits & DEV_CAPACITY) s += "capacity-exceeded ";
    if (s.empty()) s = "none";
    return s.c_str();
}

int splat_version(void) { return 1; }

size_t splat_project_fwd_workspace_size(const splat_params *p) {
    return p ? project_ws_bytes(*p) : 0;
}

}  // extern "C"

// splat_project_fwd, and with colors / opacities / packed non-null also the
// packed records (splat_project_fwd_packed).
static int project_fwd_entry(const splat_params *p, const float *means3d, const float *scales,
                             const float *quats, const float *viewmat, float *cov3d, float *xys,
                             float *depths, int32_t *radii, float *conics, float *compensation,
                             int32_t *num_tiles_hit, int32_t *cum_tiles_hit, int64_t *total_out,
                             void *workspace, size_t workspace_bytes, const float *colors,
                             const float *opacities, float *packed, splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->num_points == 0) {
        if (total_out && cudaMemsetAsync(total_out, 0, sizeof(int64_t), s) != cudaSuccess)
            return check_launch("total memset");
        return SPLAT_OK;
    }
    NEED(means3d); NEED(scales); NEED(quats); NEED(viewmat); NEED(cov3d); NEED(xys);
    NEED(depths); NEED(radii); NEED(conics); NEED(compensation); NEED(num_tiles_hit);
    // without cum_tiles_hit only the intersection total is produced (the
    // count-only kernel), so the total then has somewhere to go
    if (!cum_tiles_hit && !total_out)
        return fail(SPLAT_ERR_INVALID_ARG, "project_fwd needs cum_tiles_hit or total_out");
    NEED_WS(workspace);
    if (workspace_bytes < project_ws_bytes(*p))
        return fail(SPLAT_ERR_WORKSPACE, "project workspace too small: need %zu, got %zu",
                    project_ws_bytes(*p), workspace_bytes);
    Arena ar{static_cast<char *>(workspace), workspace_bytes};
    int64_t *total_slot = ar.take<int64_t>(1);
    const size_t parts = (p->num_points + 255) / 256;
    unsigned long long *words = ar.take<unsigned long long>(parts + 1);
    return launch_project_fwd(*p, means3d, scales, quats, viewmat, cov3d, xys, depths, radii,
                              conics, compensation, num_tiles_hit, cum_tiles_hit,
                              total_out ? total_out : total_slot, words, colors, opacities,
                              packed, s);
}

extern "C" {

int splat_project_fwd(const splat_params *p, const float *means3d, const float *scales,
                      const float *quats, const float *viewmat, float *cov3d, float *xys,
                      float *depths, int32_t *radii, float *conics, float *compensation,
                      int32_t *num_tiles_hit, int32_t *cum_tiles_hit, int64_t *total_out,
                      void *workspace, size_t workspace_bytes, splat_stream_t stream) {
    return project_fwd_entry(p, means3d, scales, quats, viewmat, cov3d, xys, depths, radii,
                             conics, compensation, num_tiles_hit, cum_tiles_hit, total_out,
                             workspace, workspace_bytes, nullptr, nullptr, nullptr, stream);
}

int splat_project_fwd_packed(const splat_params *p, const float *means3d, const float *scales,
                             const float *quats, const float *viewmat, const float *colors,
                             const float *opacities, float *cov3d, float *xys, float *depths,
                             int32_t *radii, float *conics, float *compensation,
                             int32_t *num_tiles_hit, int32_t *cum_tiles_hit, int64_t *total_out,
                             float *packed, void *workspace, size_t workspace_bytes,
                             splat_stream_t stream) {
    if (p && p->num_points > 0) {
        NEED(colors); NEED(opacities); NEED(packed);
        if (reinterpret_cast<uintptr_t>(packed) % 16)
            return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    }
    return project_fwd_entry(p, means3d, scales, quats, viewmat, cov3d, xys, depths, radii,
                             conics, compensation, num_tiles_hit, cum_tiles_hit, total_out,
                             workspace, workspace_bytes, colors, opacities, packed, stream);
}

int splat_read_counts(const splat_params *p, const int32_t *cum_tiles_hit,
                      const int64_t *total_dev, uint32_t *status_dev, int64_t *num_intersects,
                      uint32_t *status_out, splat_stream_t stream) {
    if (!p) return fail(SPLAT_ERR_INVALID_ARG, "params is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    long long total = 0;
    uint32_t bits = 0;
    if (total_dev) {
        if (cudaMemcpyAsync(&total, total_dev, sizeof(total), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return check_launch("count read");
    } else if (p->num_points > 0) {
        NEED(cum_tiles_hit);
        int32_t v = 0;
        if (cudaMemcpyAsync(&v, cum_tiles_hit + p->num_points - 1, sizeof(v),
                            cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return check_launch("count read");
        if (cudaStreamSynchronize(s) != cudaSuccess) return check_launch("count read");
        total = v;
    }
    if (status_dev) {
        if (cudaMemcpyAsync(&bits, status_dev, sizeof(bits), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemsetAsync(status_dev, 0, sizeof(uint32_t), s) != cudaSuccess)
            return check_launch("status read");
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return check_launch("count read");
    if (num_intersects) *num_intersects = total;
    if (status_out) *status_out = bits;
    if (bits) return fail(SPLAT_ERR_DEVICE, "device status: %s", splat_device_status_string(bits));
    return check_count(total);
}

size_t splat_sort_workspace_size(const splat_params *p, int64_t num_intersects) {
    if (!p || num_intersects < 0) return 0;
    return sort_workspace_bytes(*p, num_intersects);
}

int splat_sort_and_bin(const splat_params *p, int64_t num_intersects, const int64_t *count_dev,
                       const float *xys, const float *depths, const int32_t *radii,
                       const int32_t *cum_tiles_hit, int32_t *gaussian_ids_sorted,
                       int32_t *tile_bins, int64_t *isect_ids, int32_t *gaussian_ids,
                       int64_t *isect_ids_sorted, void *workspace, size_t workspace_bytes,
                       splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_count(num_intersects)) return rc;
    NEED_BINS(tile_bins);
    if (num_intersects > 0) {
        NEED(xys); NEED(depths); NEED(radii); NEED(gaussian_ids_sorted); NEED_WS(workspace);
        if (isect_ids) NEED(cum_tiles_hit);
    }
    const Count c{reinterpret_cast<const long long *>(count_dev), num_intersects, num_intersects};
    return launch_sort_and_bin(*p, c, xys, depths, radii, cum_tiles_hit, gaussian_ids_sorted,
                               reinterpret_cast<int2 *>(tile_bins),
                               reinterpret_cast<long long *>(isect_ids), gaussian_ids,
                               reinterpret_cast<long long *>(isect_ids_sorted), workspace,
                               workspace_bytes, (cudaStream_t)stream);
}

int splat_pack_splats(const splat_params *p, const float *xys, const float *conics,
                      const float *colors, const float *opacities, float *packed,
                      splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (p->num_points == 0) return SPLAT_OK;
    NEED(xys); NEED(conics); NEED(colors); NEED(opacities); NEED(packed);
    if (reinterpret_cast<uintptr_t>(packed) % 16 || reinterpret_cast<uintptr_t>(xys) % 8)
        return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte and xys 8-byte aligned");
    return launch_pack(*p, xys, conics, colors, opacities, packed, (cudaStream_t)stream);
}

int splat_rasterize_fwd(const splat_params *p, int64_t num_intersects, const int64_t *count_dev,
                        const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                        const float *packed, const float *background, float *final_Ts,
                        int32_t *final_idx, float *out_img, uint8_t *blend_out,
                        splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_count(num_intersects)) return rc;
    NEED(background); NEED(final_Ts); NEED(final_idx); NEED(out_img);
    if (num_intersects > 0) {
        NEED(gaussian_ids_sorted); NEED_BINS(tile_bins); NEED(packed);
        if (reinterpret_cast<uintptr_t>(packed) % 16)
            return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    }
    const Count c{reinterpret_cast<const long long *>(count_dev), num_intersects, num_intersects};
    return launch_raster_fwd(*p, c, gaussian_ids_sorted,
                             reinterpret_cast<const int2 *>(tile_bins), packed, background,
                             final_Ts, final_idx, out_img, nullptr, nullptr, nullptr,
                             p->block_width == 16 ? blend_out : nullptr, (cudaStream_t)stream);
}

int splat_rasterize_fwd_l2(const splat_params *p, int64_t num_intersects, const int64_t *count_dev,
                           const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                           const float *packed, const float *background, const float *target,
                           float *final_Ts, int32_t *final_idx, float *out_img, float *v_img,
                           float *loss_out, uint8_t *blend_out, splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_count(num_intersects)) return rc;
    NEED(background); NEED(target); NEED(final_Ts); NEED(final_idx); NEED(out_img);
    NEED(v_img); NEED(loss_out);
    if (num_intersects > 0) {
        NEED(gaussian_ids_sorted); NEED_BINS(tile_bins); NEED(packed);
        if (reinterpret_cast<uintptr_t>(packed) % 16)
            return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    }
    const Count c{reinterpret_cast<const long long *>(count_dev), num_intersects, num_intersects};
    return launch_raster_fwd(*p, c, gaussian_ids_sorted,
                             reinterpret_cast<const int2 *>(tile_bins), packed, background,
                             final_Ts, final_idx, out_img, target, v_img, loss_out,
                             p->block_width == 16 ? blend_out : nullptr, (cudaStream_t)stream);
}

int splat_count_pairs(const splat_params *p, int64_t num_intersects, const int64_t *count_dev,
                      const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                      const float *packed, const int32_t *final_idx, uint64_t *counts,
                      splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_count(num_intersects)) return rc;
    NEED(counts);
    if (num_intersects > 0) {
        NEED(gaussian_ids_sorted); NEED_BINS(tile_bins); NEED(packed); NEED(final_idx);
        if (reinterpret_cast<uintptr_t>(packed) % 16)
            return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    }
    const Count c{reinterpret_cast<const long long *>(count_dev), num_intersects, num_intersects};
    return launch_count_pairs(*p, c, gaussian_ids_sorted, reinterpret_cast<const int2 *>(tile_bins),
                              packed, final_idx, reinterpret_cast<unsigned long long *>(counts),
                              (cudaStream_t)stream);
}

int splat_rasterize_bwd(const splat_params *p, int64_t num_intersects, const int64_t *count_dev,
                        const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                        const float *packed, const float *background, const float *final_Ts,
                        const int32_t *final_idx, const float *v_img, const float *v_img_alpha,
                        float *v_colors, float *v_opacity, float *v_xy, float *v_xy_abs,
                        float *v_conic, const uint8_t *blend, splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_count(num_intersects)) return rc;
    if (p->num_points > 0) {
        NEED(v_colors); NEED(v_opacity); NEED(v_xy); NEED(v_conic);
    }
    if (num_intersects > 0) {
        NEED(gaussian_ids_sorted); NEED_BINS(tile_bins); NEED(packed); NEED(background);
        NEED(final_Ts); NEED(final_idx); NEED(v_img); NEED(v_img_alpha);
        if (reinterpret_cast<uintptr_t>(packed) % 16)
            return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    }
    const Count c{reinterpret_cast<const long long *>(count_dev), num_intersects, num_intersects};
    return launch_raster_bwd(*p, c, gaussian_ids_sorted,
                             reinterpret_cast<const int2 *>(tile_bins), packed, background,
                             final_Ts, final_idx, v_img, v_img_alpha, v_colors, v_opacity, v_xy,
                             v_xy_abs, v_conic, p->block_width == 16 ? blend : nullptr,
                             (cudaStream_t)stream);
}

int splat_project_bwd(const splat_params *p, const float *means3d, const float *scales,
                      const float *quats, const float *viewmat, const float *cov3d,
                      const int32_t *radii, const float *conics, const float *compensation,
                      const float *v_xy, const float *v_depth, const float *v_conic,
                      const float *v_compensation, float *v_mean3d, float *v_scale,
                      float *v_quat, float *v_cov2d, float *v_cov3d, splat_stream_t stream) {
    if (int rc = validate(p)) return rc;
    if (p->num_points == 0) return SPLAT_OK;
    NEED(means3d); NEED(scales); NEED(quats); NEED(viewmat); NEED(cov3d); NEED(radii);
    NEED(conics); NEED(compensation); NEED(v_xy); NEED(v_depth); NEED(v_conic);
    NEED(v_compensation); NEED(v_mean3d); NEED(v_scale); NEED(v_quat);  // v_cov2d, v_cov3d optional
    return launch_project_bwd(*p, means3d, scales, quats, viewmat, cov3d, radii, conics,
                              compensation, v_xy, v_depth, v_conic, v_compensation, v_mean3d,
                              v_scale, v_quat, v_cov2d, v_cov3d, (cudaStream_t)stream);
}

int splat_l2_loss(const float *img, const float *target, int64_t count, float *loss_out,
                  float *v_img, splat_stream_t stream) {
    if (count <= 0) return fail(SPLAT_ERR_INVALID_ARG, "count must be positive");
    NEED(img); NEED(target); NEED(loss_out); NEED(v_img);
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(loss_out, 0, sizeof(float), s) != cudaSuccess) return check_launch("loss memset");
    long long blocks = (count + 255) / 256;
    if (blocks > 152 * 4) blocks = 152 * 4;
    l2_loss_kernel<<<(unsigned)blocks, 256, 0, s>>>(img, target, count, 1.f / (float)count,
                                                   loss_out, v_img);
    return check_launch("l2_loss_kernel");
}

int splat_selftest_wait_timeout(uint32_t limit, uint32_t *status_dev, splat_stream_t stream) {
    NEED(status_dev);
    if (limit == 0 || limit > (1u << 20))
        return fail(SPLAT_ERR_INVALID_ARG, "limit must be in [1, 2^20]");
    wait_timeout_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(limit, status_dev);
    return check_launch("wait_timeout_kernel");
}

int splat_xla_make_descriptor(uint32_t num_points, uint32_t img_h, uint32_t img_w, float fx,
                              float fy, float cx, float cy, float glob_scale, float clip_thresh,
                              uint32_t block_width, void *out, size_t out_len) {
    if (!out || out_len < sizeof(XlaDescriptor))
        return fail(SPLAT_ERR_INVALID_ARG, "descriptor buffer must hold %zu bytes",
                    sizeof(XlaDescriptor));
    if (block_width == 0) return fail(SPLAT_ERR_INVALID_ARG, "block_width must be positive");
    XlaDescriptor d;
    std::memset(&d, 0, sizeof(d));
    d.num_points = num_points;
    d.img_shape[0] = img_w;
    d.img_shape[1] = img_h;
    d.img_shape[2] = 1;
    d.intrins[0] = fx; d.intrins[1] = fy; d.intrins[2] = cx; d.intrins[3] = cy;
    d.glob_scale = glob_scale;
    d.clip_thresh = clip_thresh;
    d.block_width = block_width;
    d.block_dim_1d = block_width * block_width;
    d.grid_dim_1d = (num_points + d.block_dim_1d - 1) / d.block_dim_1d;
    d.grid_dim_2d[0] = (img_w + block_width - 1) / block_width;
    d.grid_dim_2d[1] = (img_h + block_width - 1) / block_width;
    d.grid_dim_2d[2] = 1;
    d.block_dim_2d[0] = block_width;
    d.block_dim_2d[1] = block_width;
    d.block_dim_2d[2] = 1;
    std::memcpy(out, &d, sizeof(d));
    return SPLAT_OK;
}

// Legacy custom calls -------------------------------------------------------

void splat_xla_project_fwd(splat_stream_t stream, void **b, const char *opaque, size_t len) {
    splat_params p;
    int rc = unpack(opaque, len, &p);
    if (rc == SPLAT_OK) {
        cudaStream_t s = (cudaStream_t)stream;
        const size_t ws_bytes = project_ws_bytes(p);
        void *ws = nullptr;
        if (cudaMallocAsync(&ws, ws_bytes, s) != cudaSuccess) {
            rc = check_launch("workspace allocation");
        } else {
            rc = splat_project_fwd(&p, (const float *)b[0], (const float *)b[1],
                                   (const float *)b[2], (const float *)b[3], (float *)b[4],
                                   (float *)b[5], (float *)b[6], (int32_t *)b[7], (float *)b[8],
                                   (float *)b[9], (int32_t *)b[10], (int32_t *)b[11], nullptr, ws,
                                   ws_bytes, stream);
            cudaFreeAsync(ws, s);
        }
    }
    report("project_fwd", rc);
}

void splat_xla_project_bwd(splat_stream_t stream, void **b, const char *opaque, size_t len) {
    splat_params p;
    int rc = unpack(opaque, len, &p);
    if (rc == SPLAT_OK)
        rc = splat_project_bwd(&p, (const float *)b[0], (const float *)b[1], (const float *)b[2],
                               (const float *)b[3], (const float *)b[4], (const int32_t *)b[6],
                               (const float *)b[7], (const float *)b[8], (const float *)b[10],
                               (const float *)b[11], (const float *)b[12], (const float *)b[9],
                               (float *)b[13], (float *)b[14], (float *)b[15], (float *)b[16],
                               (float *)b[17], stream);
    report("project_bwd", rc);
}

// Shared by the two rasterize custom calls: count, allocate, sort and bin.
struct SortedList {
    long long count = 0;
    int32_t *ids = nullptr;
    int32_t *bins = nullptr;
    float *packed = nullptr;
    void *ws = nullptr;
};

static int xla_sorted(const splat_params &p, void **b, cudaStream_t s, SortedList &L) {
    const int32_t *cum = (const int32_t *)b[7];
    if (int rc = read_count(cum, p.num_points, &L.count, s)) return rc;
    const size_t ntiles = n_tiles(p);
    const size_t ws_bytes = sort_workspace_bytes(p, L.count);
    if (cudaMallocAsync((void **)&L.bins, sizeof(int32_t) * 2 * ntiles, s) != cudaSuccess ||
        cudaMallocAsync((void **)&L.ids, sizeof(int32_t) * (size_t)(L.count ? L.count : 1), s) != cudaSuccess ||
        cudaMallocAsync((void **)&L.packed, sizeof(float) * 12 * (size_t)(p.num_points ? p.num_points : 1), s) != cudaSuccess ||
        cudaMallocAsync(&L.ws, ws_bytes, s) != cudaSuccess)
        return check_launch("sort buffer allocation");
    // colors b[0], opacities b[1], xys b[3], conics b[6]
    if (int rc = splat_pack_splats(&p, (const float *)b[3], (const float *)b[6], (const float *)b[0],
                                   (const float *)b[1], L.packed, (splat_stream_t)s))
        return rc;
    return splat_sort_and_bin(&p, L.count, nullptr, (const float *)b[3], (const float *)b[4],
                              (const int32_t *)b[5], cum, L.ids, L.bins, nullptr, nullptr,
                              nullptr, L.ws, ws_bytes, (splat_stream_t)s);
}

static void xla_release(SortedList &L, cudaStream_t s) {
    if (L.ids) cudaFreeAsync(L.ids, s);
    if (L.bins) cudaFreeAsync(L.bins, s);
    if (L.packed) cudaFreeAsync(L.packed, s);
    if (L.ws) cudaFreeAsync(L.ws, s);
}

void splat_xla_rasterize_fwd(splat_stream_t stream, void **b, const char *opaque, size_t len) {
    splat_params p;
    int rc = unpack(opaque, len, &p);
    if (rc == SPLAT_OK) {
        cudaStream_t s = (cudaStream_t)stream;
        SortedList L;
        rc = xla_sorted(p, b, s, L);
        if (rc == SPLAT_OK)
            rc = splat_rasterize_fwd(&p, L.count, nullptr, L.ids, L.bins, L.packed, (const float *)b[2],
                                     (float *)b[8], (int32_t *)b[9], (float *)b[10], nullptr,
                                     stream);
        xla_release(L, s);
    }
    report("rasterize_fwd", rc);
}

void splat_xla_rasterize_bwd(splat_stream_t stream, void **b, const char *opaque, size_t len) {
    splat_params p;
    int rc = unpack(opaque, len, &p);
    if (rc == SPLAT_OK) {
        cudaStream_t s = (cudaStream_t)stream;
        SortedList L;
        rc = xla_sorted(p, b, s, L);
        if (rc == SPLAT_OK)
            rc = splat_rasterize_bwd(&p, L.count, nullptr, L.ids, L.bins, L.packed, (const float *)b[2],
                                     (const float *)b[8], (const int32_t *)b[9],
                                     (const float *)b[10], (const float *)b[11], (float *)b[12],
                                     (float *)b[13], (float *)b[14], (float *)b[15],
                                     (float *)b[16], nullptr, stream);
        xla_release(L, s);
    }
    report("rasterize_bwd", rc);
}

}  // extern "C"
