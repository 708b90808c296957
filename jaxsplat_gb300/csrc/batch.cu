// batch.cu -- many views of several scenes through one pass of each kernel.
//
// An entry is a (view, Gaussian) pair; view v's entries occupy
// [entry_base, entry_base + num_points) rounded up to a multiple of 256, so a
// 256-thread block of the per-entry kernels belongs to one view.  The sort
// (sort.cu) and the rasterizers (raster.cu) run over all entries, all tiles
// and all pixels at once; this file holds the per-entry projection, the
// per-view loss and the projection backward, whose scene gradients are
// summed over the views with atomics, and the batch entry points.
#include <algorithm>

#include "project_math.cuh"
#include "splat_internal.cuh"

namespace splat {

constexpr int kBatchBlock = 256;

struct BatchProjArgs {
    const splat_view *views;
    int nviews;
    unsigned long long entries;
    float glob_scale, clip;
    unsigned bw;
    const float *means3d, *scales, *quats;
    float *cov3d, *xys, *depths, *conics, *comp;
    int32_t *radii;
    unsigned long long *total;
    // optional (rec non-null): each entry's packed record, as
    // splat_batch_pack writes it (colour and opacity of the scene Gaussian)
    const float *colors, *opac;
    float4 *rec;
};

__device__ __forceinline__ ProjCam view_cam(const splat_view &v, float glob, float clip,
                                            unsigned bw) {
    // forward.cu:70-71: tan_fov evaluated in double, rounded to float
    return ProjCam{v.viewmat,
                   glob,
                   v.fx,
                   v.fy,
                   v.cx,
                   v.cy,
                   (float)(0.5 * (double)v.img_width / (double)v.fx),
                   (float)(0.5 * (double)v.img_height / (double)v.fy),
                   clip,
                   v.tiles_x,
                   v.tiles_y,
                   bw};
}

__global__ void __launch_bounds__(kBatchBlock) batch_project_fwd_kernel(BatchProjArgs a) {
    __shared__ unsigned s_hits[kBatchBlock / 32];
    __shared__ ProjCam s_cam;
    __shared__ uint32_t s_base, s_gbase, s_npts;
    const size_t i = (size_t)blockIdx.x * kBatchBlock + threadIdx.x;
    if (threadIdx.x == 0) {
        // the block's view (blocks never straddle views); its camera once per
        // block -- the tangents are evaluated in double, slow on this GPU
        const splat_view &v = a.views[view_by_entry(a.views, a.nviews, (uint32_t)i)];
        s_cam = view_cam(v, a.glob_scale, a.clip, a.bw);
        s_base = v.entry_base;
        s_gbase = v.gauss_base;
        s_npts = v.num_points;
    }
    __syncthreads();
    const uint32_t k = (uint32_t)(i - s_base);
    uint32_t hits = 0;
    if (i < a.entries) {
        ProjOut o;
        if (k < s_npts) {
            const size_t g = (size_t)s_gbase + k;
            o = project_one(s_cam, a.means3d + 3 * g, a.scales + 3 * g, a.quats + 4 * g);
        } else {  // padding: a culled Gaussian
#pragma unroll
            for (int q = 0; q < 6; ++q) o.cov[q] = 0.f;
            o.conic = make_float3(0.f, 0.f, 0.f);
            o.center = make_float2(0.f, 0.f);
            o.depth = o.comp = 0.f;
            o.radius = 0;
            o.hits = 0;
        }
        hits = o.hits;
#pragma unroll
        for (int q = 0; q < 6; ++q) a.cov3d[6 * i + q] = o.cov[q];
        a.xys[2 * i] = o.center.x;
        a.xys[2 * i + 1] = o.center.y;
        a.depths[i] = o.depth;
        a.radii[i] = o.radius;
        a.conics[3 * i] = o.conic.x;
        a.conics[3 * i + 1] = o.conic.y;
        a.conics[3 * i + 2] = o.conic.z;
        a.comp[i] = o.comp;
        if (a.rec) {
            float4 *r = a.rec + 3 * i;
            if (k < s_npts) {
                const size_t g = (size_t)s_gbase + k;
                write_record(r, o.center, o.conic, a.opac[g],
                             make_float3(a.colors[3 * g], a.colors[3 * g + 1], a.colors[3 * g + 2]),
                             __int_as_float((int)g));
            } else {  // padding: a record that no pixel passes (pack_batch_kernel's)
                r[0] = make_float4(0.f, 0.f, 0.f, 0.f);
                r[1] = make_float4(0.f, 0.f, 0.f, 0.f);
                r[2] = make_float4(0.f, -CUDART_INF_F, -CUDART_INF_F, __int_as_float((int)s_gbase));
            }
        }
    }
    // block total of the tile counts -> one atomic per block
    unsigned w = hits;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) w += __shfl_xor_sync(0xffffffffu, w, off);
    if ((threadIdx.x & 31) == 0) s_hits[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int q = 0; q < kBatchBlock / 32; ++q) t += s_hits[q];
        if (t) atomicAdd(a.total, t);
    }
}

// Per-view mean squared error: weight 1 / (3 H W) for the view's pixels.
__global__ void batch_l2_kernel(const splat_view *views, int nviews, unsigned long long npix,
                                const float *img, const float *target, float *loss,
                                float *v_img) {
    float local = 0.f;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long p = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         p < npix; p += stride) {
        const splat_view &v = views[view_by_pixel(views, nviews, p)];
        const float inv = 1.f / (3.f * (float)v.img_width * (float)v.img_height);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float d = img[3 * p + c] - target[3 * p + c];
            v_img[3 * p + c] = 2.f * d * inv;
            local += d * d * inv;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    __shared__ float s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        float x = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (threadIdx.x == 0) atomicAdd(loss, x);
    }
}

struct BatchProjBwdArgs {
    const splat_view *views;
    int nviews;
    unsigned long long entries;
    float glob_scale;
    const float *means3d, *scales, *quats;
    const float *cov3d, *conics, *comp, *v_xy, *v_conic;
    const int32_t *radii;
    float *v_mean3d, *v_scale, *v_quat;
};

__global__ void __launch_bounds__(kBatchBlock) batch_project_bwd_kernel(BatchProjBwdArgs a) {
    const size_t i = (size_t)blockIdx.x * kBatchBlock + threadIdx.x;
    if (i >= a.entries || a.radii[i] <= 0) return;
    const splat_view &v = a.views[view_by_entry(a.views, a.nviews, (uint32_t)i)];
    const uint32_t k = (uint32_t)(i - v.entry_base);
    if (k >= v.num_points) return;
    const size_t g = (size_t)v.gauss_base + k;
    const ProjCam cam{v.viewmat, a.glob_scale, v.fx, v.fy, 0.f, 0.f, 0.f, 0.f, 0.f, 0u, 0u, 0u};
    // render's zero cotangents for depth and compensation (jaxsplat/__init__.py:6-70)
    const ProjVjp r = project_vjp_one(cam, a.means3d + 3 * g, a.scales + 3 * g, a.quats + 4 * g,
                                      a.cov3d + 6 * i, a.conics + 3 * i, a.comp[i],
                                      a.v_xy + 2 * i, 0.f, a.v_conic + 3 * i, 0.f);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        atomicAdd(&a.v_mean3d[3 * g + q], r.vmean[q]);
        atomicAdd(&a.v_scale[3 * g + q], r.vscale[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) atomicAdd(&a.v_quat[4 * g + q], r.vquat[q]);
}

// Launchers in sort.cu and raster.cu.
size_t batch_sort_workspace_bytes(const splat_batch &, long long);
int launch_batch_sort_and_bin(const splat_batch &, Count, const float *, const float *,
                              const int32_t *, int32_t *, int2 *, int32_t *, void *, size_t,
                              cudaStream_t);
int launch_batch_pack(const splat_batch &, const float *, const float *, const float *,
                      const float *, float *, cudaStream_t);
int launch_batch_raster_fwd(const splat_batch &, Count, const int32_t *, const int2 *,
                            const int32_t *, const float *, float *, int32_t *, float *,
                            const float *, float *, float *, int, int *, cudaStream_t);
int launch_batch_raster_bwd(const splat_batch &, Count, const int32_t *, const int2 *,
                            const int32_t *, const float *, const float *, const int32_t *,
                            const float *, const float *, float *, float *, float *, float *, int,
                            int *, cudaStream_t);

static int check_batch(const splat_batch *b) {
    if (!b) return fail(SPLAT_ERR_INVALID_ARG, "batch is NULL");
    if (!b->views || b->num_views == 0 || b->num_scenes == 0)
        return fail(SPLAT_ERR_INVALID_ARG, "batch needs a device view table and at least one view");
    if (b->block_width < 2 || b->block_width > 16)
        return fail(SPLAT_ERR_INVALID_ARG, "block_width must be in [2, 16], got %u", b->block_width);
    if (b->num_entries > 0x7fffffffull || b->num_tiles > 0x7fffffffull ||
        b->num_points > 0x7fffffffull)
        return fail(SPLAT_ERR_OVERFLOW, "batch exceeds 2^31 entries, tiles or Gaussians");
    if (b->num_entries == 0 && b->num_tiles == 0)
        return fail(SPLAT_ERR_INVALID_ARG, "batch totals are zero: call splat_batch_layout first");
    return SPLAT_OK;
}

static int check_capacity(int64_t capacity) {
    if (capacity < 0 || capacity > (int64_t)(1u << 30) - 1)
        return fail(SPLAT_ERR_OVERFLOW, "capacity %lld outside [0, 2^30 - 1]", (long long)capacity);
    return SPLAT_OK;
}

}  // namespace splat

using namespace splat;

#define NEED(ptr)                                                                       \
    do {                                                                                \
        if (!(ptr)) return fail(SPLAT_ERR_INVALID_ARG, "%s must not be NULL", #ptr);   \
    } while (0)

// tile_bins is read and written as int2
#define NEED_BINS(ptr)                                                                     \
    do {                                                                                   \
        NEED(ptr);                                                                         \
        if (reinterpret_cast<uintptr_t>(ptr) % 8)                                          \
            return fail(SPLAT_ERR_INVALID_ARG, "%s must be 8-byte aligned", #ptr);         \
    } while (0)

extern "C" {

int splat_batch_layout(splat_batch *b, splat_view *views, const uint32_t *scene_points) {
    NEED(b);
    NEED(views);
    NEED(scene_points);
    if (b->num_views == 0 || b->num_scenes == 0)
        return fail(SPLAT_ERR_INVALID_ARG, "batch needs at least one scene and one view");
    if (b->block_width < 2 || b->block_width > 16)
        return fail(SPLAT_ERR_INVALID_ARG, "block_width must be in [2, 16], got %u", b->block_width);
    unsigned long long gauss = 0;
    for (uint32_t s = 0; s < b->num_scenes; ++s) gauss += scene_points[s];
    // Gaussian ids (the sorted lists, the records' scene-index tag) are int32
    if (gauss > 0x7fffffffull)
        return fail(SPLAT_ERR_OVERFLOW, "scenes hold %llu Gaussians in total, more than 2^31 - 1",
                    gauss);
    unsigned long long entry = 0, tile = 0, pix = 0;
    for (uint32_t k = 0; k < b->num_views; ++k) {
        splat_view &v = views[k];
        if (v.scene >= b->num_scenes)
            return fail(SPLAT_ERR_INVALID_ARG, "view %u names scene %u of %u", k, v.scene,
                        b->num_scenes);
        if (v.img_width == 0 || v.img_height == 0 || !(v.fx > 0.f) || !(v.fy > 0.f))
            return fail(SPLAT_ERR_INVALID_ARG, "view %u: empty image or non-positive focal length", k);
        unsigned long long base = 0;
        for (uint32_t s = 0; s < v.scene; ++s) base += scene_points[s];
        v.gauss_base = (uint32_t)base;
        v.num_points = scene_points[v.scene];
        v.tiles_x = (v.img_width + b->block_width - 1) / b->block_width;
        v.tiles_y = (v.img_height + b->block_width - 1) / b->block_width;
        v.entry_base = (uint32_t)entry;
        v.tile_base = (uint32_t)tile;
        v.pixel_base = pix;
        entry += ((unsigned long long)v.num_points + kBatchBlock - 1) / kBatchBlock * kBatchBlock;
        tile += (unsigned long long)v.tiles_x * v.tiles_y;
        pix += (unsigned long long)v.img_width * v.img_height;
        if (entry > 0x7fffffffull || tile > 0x7fffffffull)
            return fail(SPLAT_ERR_OVERFLOW, "batch exceeds 2^31 entries or tiles at view %u", k);
    }
    b->num_points = gauss;
    b->num_entries = entry;
    b->num_tiles = tile;
    b->num_pixels = pix;
    return SPLAT_OK;
}

}  // extern "C"

static int batch_project_entry(const splat_batch *b, const float *means3d, const float *scales,
                               const float *quats, const float *colors, const float *opacities,
                               float *cov3d, float *xys, float *depths, int32_t *radii,
                               float *conics, float *compensation, int64_t *total_dev,
                               float *packed, splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    NEED(total_dev);
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(total_dev, 0, sizeof(int64_t), s) != cudaSuccess)
        return check_launch("batch total memset");
    if (b->num_entries == 0) return SPLAT_OK;
    NEED(means3d); NEED(scales); NEED(quats); NEED(cov3d); NEED(xys); NEED(depths);
    NEED(radii); NEED(conics); NEED(compensation);
    BatchProjArgs a;
    a.views = b->views;
    a.nviews = (int)b->num_views;
    a.entries = b->num_entries;
    a.glob_scale = b->glob_scale;
    a.clip = b->clip_thresh;
    a.bw = b->block_width;
    a.means3d = means3d; a.scales = scales; a.quats = quats;
    a.cov3d = cov3d; a.xys = xys; a.depths = depths; a.conics = conics; a.comp = compensation;
    a.radii = radii;
    a.total = reinterpret_cast<unsigned long long *>(total_dev);
    a.colors = colors; a.opac = opacities; a.rec = reinterpret_cast<float4 *>(packed);
    batch_project_fwd_kernel<<<(unsigned)(b->num_entries / kBatchBlock), kBatchBlock, 0, s>>>(a);
    return check_launch("batch_project_fwd_kernel");
}

extern "C" {

int splat_batch_project_fwd(const splat_batch *b, const float *means3d, const float *scales,
                            const float *quats, float *cov3d, float *xys, float *depths,
                            int32_t *radii, float *conics, float *compensation,
                            int64_t *total_dev, splat_stream_t stream) {
    return batch_project_entry(b, means3d, scales, quats, nullptr, nullptr, cov3d, xys, depths,
                               radii, conics, compensation, total_dev, nullptr, stream);
}

int splat_batch_project_fwd_packed(const splat_batch *b, const float *means3d,
                                   const float *scales, const float *quats, const float *colors,
                                   const float *opacities, float *cov3d, float *xys,
                                   float *depths, int32_t *radii, float *conics,
                                   float *compensation, int64_t *total_dev, float *packed,
                                   splat_stream_t stream) {
    if (b && b->num_entries > 0) {
        NEED(colors); NEED(opacities); NEED(packed);
        if (reinterpret_cast<uintptr_t>(packed) % 16)
            return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    }
    return batch_project_entry(b, means3d, scales, quats, colors, opacities, cov3d, xys, depths,
                               radii, conics, compensation, total_dev, packed, stream);
}

size_t splat_batch_sort_workspace_size(const splat_batch *b, int64_t capacity) {
    if (check_batch(b) || check_capacity(capacity)) return 0;
    return batch_sort_workspace_bytes(*b, capacity);
}

int splat_batch_sort_and_bin(const splat_batch *b, int64_t capacity, const int64_t *count_dev,
                             const float *xys, const float *depths, const int32_t *radii,
                             int32_t *gaussian_ids_sorted, int32_t *tile_bins,
                             int32_t *tile_order, void *workspace, size_t workspace_bytes,
                             splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    if (int rc = check_capacity(capacity)) return rc;
    NEED(count_dev); NEED(xys); NEED(depths); NEED(radii); NEED_BINS(tile_bins); NEED(tile_order);
    NEED(workspace);
    // 64-bit look-back words updated by atomics: 256-byte aligned, as every
    // device allocator returns it
    if (reinterpret_cast<uintptr_t>(workspace) % 256)
        return fail(SPLAT_ERR_INVALID_ARG, "workspace must be 256-byte aligned");
    if (capacity > 0) NEED(gaussian_ids_sorted);
    const Count c{reinterpret_cast<const long long *>(count_dev), 0, capacity};
    return launch_batch_sort_and_bin(*b, c, xys, depths, radii, gaussian_ids_sorted,
                                     reinterpret_cast<int2 *>(tile_bins), tile_order, workspace,
                                     workspace_bytes, (cudaStream_t)stream);
}

int splat_batch_pack(const splat_batch *b, const float *xys, const float *conics,
                     const float *colors, const float *opacities, float *packed,
                     splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    NEED(xys); NEED(conics); NEED(colors); NEED(opacities); NEED(packed);
    if (reinterpret_cast<uintptr_t>(packed) % 16)
        return fail(SPLAT_ERR_INVALID_ARG, "packed must be 16-byte aligned");
    return launch_batch_pack(*b, xys, conics, colors, opacities, packed, (cudaStream_t)stream);
}

int splat_batch_rasterize_fwd(const splat_batch *b, int64_t capacity, const int64_t *count_dev,
                              const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                              const int32_t *tile_order, const float *packed, float *final_Ts,
                              int32_t *final_idx, float *out_img, uint32_t chunk,
                              int32_t *work_counter, splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    if (int rc = check_capacity(capacity)) return rc;
    NEED(count_dev); NEED_BINS(tile_bins); NEED(tile_order); NEED(packed); NEED(final_Ts);
    NEED(final_idx); NEED(out_img); NEED(work_counter);
    if (capacity > 0) NEED(gaussian_ids_sorted);
    if (chunk < 1 || chunk > 64) return fail(SPLAT_ERR_INVALID_ARG, "chunk must be in [1, 64]");
    const Count c{reinterpret_cast<const long long *>(count_dev), 0, capacity};
    return launch_batch_raster_fwd(*b, c, gaussian_ids_sorted,
                                   reinterpret_cast<const int2 *>(tile_bins), tile_order, packed,
                                   final_Ts, final_idx, out_img, nullptr, nullptr, nullptr,
                                   (int)chunk, work_counter, (cudaStream_t)stream);
}

int splat_batch_rasterize_fwd_l2(const splat_batch *b, int64_t capacity, const int64_t *count_dev,
                                 const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                                 const int32_t *tile_order, const float *packed,
                                 const float *target, float *final_Ts, int32_t *final_idx,
                                 float *out_img, float *v_img, float *loss_out, uint32_t chunk,
                                 int32_t *work_counter, splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    if (int rc = check_capacity(capacity)) return rc;
    NEED(count_dev); NEED_BINS(tile_bins); NEED(tile_order); NEED(packed); NEED(target);
    NEED(final_Ts); NEED(final_idx); NEED(out_img); NEED(v_img); NEED(loss_out);
    NEED(work_counter);
    if (capacity > 0) NEED(gaussian_ids_sorted);
    if (chunk < 1 || chunk > 64) return fail(SPLAT_ERR_INVALID_ARG, "chunk must be in [1, 64]");
    const Count c{reinterpret_cast<const long long *>(count_dev), 0, capacity};
    return launch_batch_raster_fwd(*b, c, gaussian_ids_sorted,
                                   reinterpret_cast<const int2 *>(tile_bins), tile_order, packed,
                                   final_Ts, final_idx, out_img, target, v_img, loss_out,
                                   (int)chunk, work_counter, (cudaStream_t)stream);
}

int splat_batch_rasterize_bwd(const splat_batch *b, int64_t capacity, const int64_t *count_dev,
                              const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                              const int32_t *tile_order, const float *packed,
                              const float *final_Ts, const int32_t *final_idx,
                              const float *v_img, const float *v_img_alpha, float *v_colors,
                              float *v_opacity, float *v_xy, float *v_conic, uint32_t chunk,
                              int32_t *work_counter, splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    if (int rc = check_capacity(capacity)) return rc;
    NEED(count_dev); NEED_BINS(tile_bins); NEED(tile_order); NEED(packed); NEED(final_Ts);
    NEED(final_idx); NEED(v_img); NEED(v_img_alpha); NEED(v_colors); NEED(v_opacity);
    NEED(v_xy); NEED(v_conic); NEED(work_counter);
    if (capacity > 0) NEED(gaussian_ids_sorted);
    if (chunk < 1 || chunk > 64) return fail(SPLAT_ERR_INVALID_ARG, "chunk must be in [1, 64]");
    const Count c{reinterpret_cast<const long long *>(count_dev), 0, capacity};
    return launch_batch_raster_bwd(*b, c, gaussian_ids_sorted,
                                   reinterpret_cast<const int2 *>(tile_bins), tile_order, packed,
                                   final_Ts, final_idx, v_img, v_img_alpha, v_colors, v_opacity,
                                   v_xy, v_conic, (int)chunk, work_counter, (cudaStream_t)stream);
}

int splat_batch_l2_loss(const splat_batch *b, const float *img, const float *target,
                        float *loss_out, float *v_img, splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    NEED(img); NEED(target); NEED(loss_out); NEED(v_img);
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(loss_out, 0, sizeof(float), s) != cudaSuccess)
        return check_launch("batch loss memset");
    if (b->num_pixels == 0) return SPLAT_OK;
    const unsigned long long blocks =
        std::min<unsigned long long>((b->num_pixels + 255) / 256, 152ull * 16);
    batch_l2_kernel<<<(unsigned)blocks, 256, 0, s>>>(b->views, (int)b->num_views, b->num_pixels,
                                                     img, target, loss_out, v_img);
    return check_launch("batch_l2_kernel");
}

int splat_batch_project_bwd(const splat_batch *b, const float *means3d, const float *scales,
                            const float *quats, const float *cov3d, const int32_t *radii,
                            const float *conics, const float *compensation, const float *v_xy,
                            const float *v_conic, float *v_mean3d, float *v_scale,
                            float *v_quat, splat_stream_t stream) {
    if (int rc = check_batch(b)) return rc;
    NEED(means3d); NEED(scales); NEED(quats); NEED(cov3d); NEED(radii); NEED(conics);
    NEED(compensation); NEED(v_xy); NEED(v_conic); NEED(v_mean3d); NEED(v_scale); NEED(v_quat);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t g = b->num_points;
    if (cudaMemsetAsync(v_mean3d, 0, g * 3 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_scale, 0, g * 3 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_quat, 0, g * 4 * sizeof(float), s) != cudaSuccess)
        return check_launch("batch project_bwd output memset");
    if (b->num_entries == 0) return SPLAT_OK;
    BatchProjBwdArgs a;
    a.views = b->views;
    a.nviews = (int)b->num_views;
    a.entries = b->num_entries;
    a.glob_scale = b->glob_scale;
    a.means3d = means3d; a.scales = scales; a.quats = quats;
    a.cov3d = cov3d; a.conics = conics; a.comp = compensation; a.v_xy = v_xy;
    a.v_conic = v_conic; a.radii = radii;
    a.v_mean3d = v_mean3d; a.v_scale = v_scale; a.v_quat = v_quat;
    batch_project_bwd_kernel<<<(unsigned)(b->num_entries / kBatchBlock), kBatchBlock, 0, s>>>(a);
    return check_launch("batch_project_bwd_kernel");
}

}  // extern "C"
