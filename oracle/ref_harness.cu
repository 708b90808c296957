// ref_harness.cu -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
//
// Drives the reference's own CUDA kernels, built unmodified from
// lib/kernels/{forward,backward,other}.cu into cubins under oracle/_ref/ by
// oracle/build.py, so that tests and bench.py's reference arm can run the
// reference on the same GPU without jax.  The cubins are loaded with the
// driver API; kernels are looked up by their (mangled) names.
//
// The four ref_xla_* entry points keep the reference's legacy XLA custom-call
// signature (lib/ops.h:45-92: stream, buffers in operand-then-result order,
// the 80-byte opaque descriptor) and repeat the host orchestration of
// lib/ops.cu step for step -- the zeroing memsets, the blocking stream
// synchronisations, the pageable device->host read of the intersection count,
// cudaMalloc/cudaFree of temporaries and CUB workspaces, CUB InclusiveSum and
// SortPairs over bits [0, 32+msb) -- so that its timing is the reference's
// stock code path.  The ref_stage_* entry points expose the intermediates
// (unsorted/sorted keys, sorted ids, tile bins) that lib/ops.cu keeps internal.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <cstdio>
#include <cstring>
#include <string>

namespace {

// Same field order and layout as ops::Descriptor (lib/ops.h:9-22).
struct RefDescriptor {
    unsigned num_points;
    dim3 img_shape;
    float4 intrins;
    float glob_scale;
    float clip_thresh;
    unsigned block_width;
    unsigned grid_dim_1d;
    unsigned block_dim_1d;
    dim3 grid_dim_2d;
    dim3 block_dim_2d;
};
static_assert(sizeof(RefDescriptor) == 80, "descriptor must be 80 bytes");

thread_local std::string g_err;

struct Kernels {
    bool loaded = false;
    CUmodule mods[3] = {nullptr, nullptr, nullptr};
    CUfunction project_fwd = nullptr, map_isect = nullptr, bin_edges = nullptr,
               raster_fwd = nullptr, raster_bwd = nullptr, project_bwd = nullptr,
               tiled_memset = nullptr;
} K;

#define HCHECK(expr)                                                           \
    do {                                                                       \
        cudaError_t e_ = (expr);                                               \
        if (e_ != cudaSuccess) {                                               \
            g_err = std::string(#expr) + ": " + cudaGetErrorString(e_);        \
            return 1;                                                          \
        }                                                                      \
    } while (0)

#define DCHECK(expr)                                                           \
    do {                                                                       \
        CUresult r_ = (expr);                                                  \
        if (r_ != CUDA_SUCCESS) {                                              \
            const char *s_ = nullptr;                                          \
            cuGetErrorString(r_, &s_);                                         \
            g_err = std::string(#expr) + ": " + (s_ ? s_ : "?");               \
            return 1;                                                          \
        }                                                                      \
    } while (0)

int find_kernel(CUmodule m, const char *needle, CUfunction *out) {
    unsigned count = 0;
    DCHECK(cuModuleGetFunctionCount(&count, m));
    CUfunction fns[64];
    if (count > 64) count = 64;
    DCHECK(cuModuleEnumerateFunctions(fns, count, m));
    for (unsigned i = 0; i < count; ++i) {
        const char *name = nullptr;
        DCHECK(cuFuncGetName(&name, fns[i]));
        if (name && std::strstr(name, needle)) {
            *out = fns[i];
            return 0;
        }
    }
    g_err = std::string("kernel not found in cubin: ") + needle;
    return 1;
}

int launch(CUfunction f, dim3 grid, dim3 block, cudaStream_t s, void **args) {
    if (grid.x == 0 || grid.y == 0 || grid.z == 0) {
        // The runtime launch in lib/ops.cu would fail with an invalid
        // configuration here; report the same failure instead of launching.
        g_err = "invalid configuration argument (empty grid)";
        return 1;
    }
    DCHECK(cuLaunchKernel(f, grid.x, grid.y, grid.z, block.x, block.y, block.z, 0,
                          (CUstream)s, args, nullptr));
    return 0;
}

// lib/ops.cu:607-643
int cumsum(cudaStream_t s, const int32_t *in, int32_t *out, int n) {
    void *ws = nullptr;
    size_t ws_bytes = 0;
    HCHECK(cub::DeviceScan::InclusiveSum(ws, ws_bytes, in, out, n, s));
    HCHECK(cudaMalloc(&ws, ws_bytes));
    HCHECK(cub::DeviceScan::InclusiveSum(ws, ws_bytes, in, out, n, s));
    HCHECK(cudaFree(ws));
    return 0;
}

int end_bit_for(const RefDescriptor &d) {
    int32_t max_tile_id = (int32_t)(d.grid_dim_2d.x * d.grid_dim_2d.y);
    int msb = 32 - __builtin_clz(max_tile_id) + 1;  // lib/ops.cu:723-724
    return 32 + msb;
}

int map_isect(cudaStream_t s, const RefDescriptor &d, const float2 *xys, const float *depths,
              const int *radii, const int *cum, int64_t *keys, int32_t *ids) {
    int num_points = (int)d.num_points;
    dim3 tile_bounds = d.grid_dim_2d;
    unsigned bw = d.block_width;
    void *args[] = {&num_points, &xys, &depths, &radii, &cum, &tile_bounds, &bw, &keys, &ids};
    return launch(K.map_isect, dim3(d.grid_dim_1d), dim3(d.block_dim_1d), s, args);
}

int sort_pairs(cudaStream_t s, unsigned count, const int64_t *kin, int64_t *kout,
               const int32_t *vin, int32_t *vout, int end_bit) {
    void *ws = nullptr;
    size_t ws_bytes = 0;
    HCHECK(cub::DeviceRadixSort::SortPairs(ws, ws_bytes, kin, kout, vin, vout, count, 0,
                                           end_bit, s));
    HCHECK(cudaMalloc(&ws, ws_bytes));
    HCHECK(cub::DeviceRadixSort::SortPairs(ws, ws_bytes, kin, kout, vin, vout, count, 0,
                                           end_bit, s));
    HCHECK(cudaFree(ws));
    return 0;
}

int bin_edges(cudaStream_t s, const RefDescriptor &d, unsigned count, const int64_t *sorted,
              int2 *bins) {
    int n = (int)count;
    void *args[] = {&n, &sorted, &bins};
    return launch(K.bin_edges, dim3((count + d.block_dim_1d - 1) / d.block_dim_1d),
                  dim3(d.block_dim_1d), s, args);
}

// lib/ops.cu:645-793
int sort_and_bin(cudaStream_t s, const RefDescriptor &d, unsigned count, const float2 *xys,
                 const float *depths, const int *radii, const int *cum, int32_t *ids_sorted,
                 int2 *bins) {
    int32_t *ids_unsorted;
    int64_t *keys_unsorted, *keys_sorted;
    HCHECK(cudaMalloc(&ids_unsorted, count * sizeof(int32_t)));
    HCHECK(cudaMemsetAsync(ids_unsorted, 0, count * sizeof(int32_t), s));
    HCHECK(cudaMalloc(&keys_unsorted, count * sizeof(int64_t)));
    HCHECK(cudaMemsetAsync(keys_unsorted, 0, count * sizeof(int64_t), s));
    HCHECK(cudaMalloc(&keys_sorted, count * sizeof(int64_t)));
    HCHECK(cudaMemsetAsync(keys_sorted, 0, count * sizeof(int64_t), s));
    if (map_isect(s, d, xys, depths, radii, cum, keys_unsorted, ids_unsorted)) return 1;
    if (sort_pairs(s, count, keys_unsorted, keys_sorted, ids_unsorted, ids_sorted,
                   end_bit_for(d)))
        return 1;
    if (bin_edges(s, d, count, keys_sorted, bins)) return 1;
    HCHECK(cudaStreamSynchronize(s));
    HCHECK(cudaFree(keys_unsorted));
    HCHECK(cudaFree(keys_sorted));
    HCHECK(cudaFree(ids_unsorted));
    HCHECK(cudaStreamSynchronize(s));
    return 0;
}

int unpack(const char *opaque, size_t len, RefDescriptor *d) {
    if (len != sizeof(RefDescriptor)) {  // lib/ffi.h:17-23
        g_err = "Invalid opaque object size";
        return 1;
    }
    std::memcpy(d, opaque, sizeof(RefDescriptor));
    if (!K.loaded) {
        g_err = "reference cubins not loaded (call ref_load first)";
        return 1;
    }
    return 0;
}

}  // namespace

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }

// Load forward.cubin, backward.cubin and other.cubin from `dir`.
int ref_load(const char *dir) {
    if (K.loaded) return 0;
    HCHECK(cudaFree(nullptr));  // make the primary context current
    const char *names[3] = {"forward.cubin", "backward.cubin", "other.cubin"};
    for (int i = 0; i < 3; ++i) {
        std::string path = std::string(dir) + "/" + names[i];
        DCHECK(cuModuleLoad(&K.mods[i], path.c_str()));
    }
    if (find_kernel(K.mods[0], "21project_gaussians_fwdE", &K.project_fwd) ||
        find_kernel(K.mods[0], "26map_gaussian_to_intersectsE", &K.map_isect) ||
        find_kernel(K.mods[0], "18get_tile_bin_edgesE", &K.bin_edges) ||
        find_kernel(K.mods[0], "13rasterize_fwdE", &K.raster_fwd) ||
        find_kernel(K.mods[1], "13rasterize_bwdE", &K.raster_bwd) ||
        find_kernel(K.mods[1], "21project_gaussians_bwdE", &K.project_bwd) ||
        find_kernel(K.mods[2], "12tiled_memsetE", &K.tiled_memset))
        return 1;
    K.loaded = true;
    return 0;
}

// lib/ffi.cu:15-52: img_shape is (H, W); dim3 holds (W, H, 1).
int ref_make_descriptor(unsigned num_points, unsigned h, unsigned w, float fx, float fy,
                        float cx, float cy, float glob_scale, float clip_thresh,
                        unsigned block_width, void *out80) {
    RefDescriptor d;
    std::memset(&d, 0, sizeof(d));
    d.num_points = num_points;
    d.img_shape = dim3(w, h, 1);
    d.intrins = make_float4(fx, fy, cx, cy);
    d.glob_scale = glob_scale;
    d.clip_thresh = clip_thresh;
    d.block_width = block_width;
    d.block_dim_1d = block_width * block_width;
    d.grid_dim_1d = (num_points + d.block_dim_1d - 1) / d.block_dim_1d;
    d.block_dim_2d = dim3(block_width, block_width, 1);
    d.grid_dim_2d = dim3((w + block_width - 1) / block_width, (h + block_width - 1) / block_width, 1);
    std::memcpy(out80, &d, sizeof(d));
    return 0;
}

// lib/ops.cu:12-61 and 237-325
int ref_xla_project_fwd(cudaStream_t s, void **b, const char *opaque, size_t len) {
    RefDescriptor d;
    if (unpack(opaque, len, &d)) return 1;
    const float3 *means = (const float3 *)b[0];
    const float3 *scales = (const float3 *)b[1];
    const float4 *quats = (const float4 *)b[2];
    const float *viewmat = (const float *)b[3];
    float *cov3d = (float *)b[4];
    float2 *xys = (float2 *)b[5];
    float *depths = (float *)b[6];
    int *radii = (int *)b[7];
    float3 *conics = (float3 *)b[8];
    float *comp = (float *)b[9];
    int *ntiles = (int *)b[10];
    int *cum = (int *)b[11];
    size_t n = d.num_points;
    HCHECK(cudaMemsetAsync(cov3d, 0, n * 6 * sizeof(float), s));
    HCHECK(cudaMemsetAsync(xys, 0, n * sizeof(float2), s));
    HCHECK(cudaMemsetAsync(depths, 0, n * sizeof(float), s));
    HCHECK(cudaMemsetAsync(radii, 0, n * sizeof(int), s));
    HCHECK(cudaMemsetAsync(conics, 0, n * sizeof(float3), s));
    HCHECK(cudaMemsetAsync(comp, 0, n * sizeof(float), s));
    HCHECK(cudaMemsetAsync(ntiles, 0, n * sizeof(int), s));
    HCHECK(cudaMemsetAsync(cum, 0, n * sizeof(int), s));
    HCHECK(cudaStreamSynchronize(s));
    int num_points = (int)d.num_points;
    float glob = d.glob_scale, clip = d.clip_thresh;
    float4 intr = d.intrins;
    dim3 img = d.img_shape, tb = d.grid_dim_2d;
    unsigned bw = d.block_width;
    void *args[] = {&num_points, &means, &scales, &glob, &quats, &viewmat, &intr, &img, &tb,
                    &bw, &clip, &cov3d, &xys, &depths, &radii, &conics, &comp, &ntiles};
    if (launch(K.project_fwd, dim3(d.grid_dim_1d), dim3(d.block_dim_1d), s, args)) return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    if (cumsum(s, ntiles, cum, num_points)) return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    return 0;
}

// lib/ops.cu:63-105 and 327-397
int ref_xla_project_bwd(cudaStream_t s, void **b, const char *opaque, size_t len) {
    RefDescriptor d;
    if (unpack(opaque, len, &d)) return 1;
    const void *means = b[0], *scales = b[1], *quats = b[2], *viewmat = b[3], *cov3d = b[4];
    /* b[5] is xys: an operand the kernel does not read */
    const void *radii = b[6], *conics = b[7], *comp = b[8], *v_comp = b[9], *v_xy = b[10],
               *v_depth = b[11], *v_conic = b[12];
    void *v_mean = b[13], *v_scale = b[14], *v_quat = b[15], *v_cov2d = b[16], *v_cov3d = b[17];
    size_t n = d.num_points;
    HCHECK(cudaMemsetAsync(v_cov2d, 0, n * 3 * sizeof(float), s));
    HCHECK(cudaMemsetAsync(v_cov3d, 0, n * 6 * sizeof(float), s));
    HCHECK(cudaMemsetAsync(v_mean, 0, n * 3 * sizeof(float), s));
    HCHECK(cudaMemsetAsync(v_scale, 0, n * 3 * sizeof(float), s));
    HCHECK(cudaMemsetAsync(v_quat, 0, n * 4 * sizeof(float), s));
    HCHECK(cudaStreamSynchronize(s));
    int num_points = (int)d.num_points;
    float glob = d.glob_scale;
    float4 intr = d.intrins;
    dim3 img = d.img_shape;
    void *args[] = {&num_points, &means, &scales, &glob, &quats, &viewmat, &intr, &img,
                    &cov3d, &radii, &conics, &comp, &v_xy, &v_depth, &v_conic, &v_comp,
                    &v_cov2d, &v_cov3d, &v_mean, &v_scale, &v_quat};
    if (launch(K.project_bwd, dim3(d.grid_dim_1d), dim3(d.block_dim_1d), s, args)) return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    return 0;
}

// lib/ops.cu:107-170 and 399-491
int ref_xla_rasterize_fwd(cudaStream_t s, void **b, const char *opaque, size_t len) {
    RefDescriptor d;
    if (unpack(opaque, len, &d)) return 1;
    const float3 *colors = (const float3 *)b[0];
    const float *opac = (const float *)b[1];
    const float3 *bg = (const float3 *)b[2];
    const float2 *xys = (const float2 *)b[3];
    const float *depths = (const float *)b[4];
    const int *radii = (const int *)b[5];
    const float3 *conics = (const float3 *)b[6];
    const int *cum = (const int *)b[7];
    float *final_Ts = (float *)b[8];
    int *final_idx = (int *)b[9];
    float3 *img = (float3 *)b[10];
    int num_isect = 0;
    HCHECK(cudaMemcpyAsync(&num_isect, cum + d.num_points - 1, sizeof(int),
                           cudaMemcpyDeviceToHost, s));
    size_t npix = (size_t)d.img_shape.x * d.img_shape.y;
    HCHECK(cudaMemsetAsync(final_Ts, 0, npix * sizeof(float), s));
    HCHECK(cudaMemsetAsync(final_idx, 0, npix * sizeof(int), s));
    HCHECK(cudaMemsetAsync(img, 0, npix * sizeof(float3), s));
    int32_t *ids_sorted = nullptr;
    int2 *bins = nullptr;
    size_t ntiles = (size_t)d.grid_dim_2d.x * d.grid_dim_2d.y;
    HCHECK(cudaMallocAsync((void **)&ids_sorted, sizeof(int32_t) * (size_t)num_isect, s));
    HCHECK(cudaMemsetAsync(ids_sorted, 0, sizeof(int32_t) * (size_t)num_isect, s));
    HCHECK(cudaMallocAsync((void **)&bins, sizeof(int2) * ntiles, s));
    HCHECK(cudaMemsetAsync(bins, 0, sizeof(int2) * ntiles, s));
    HCHECK(cudaStreamSynchronize(s));
    if (num_isect == 0) {
        float *dst = (float *)img;
        size_t ndst = npix * 3, nsrc = 3;
        const float *src = (const float *)bg;
        void *args[] = {&dst, &ndst, &src, &nsrc};
        return launch(K.tiled_memset, dim3(d.grid_dim_1d), dim3(d.block_dim_1d), s, args);
    }
    if (sort_and_bin(s, d, (unsigned)num_isect, xys, depths, radii, cum, ids_sorted, bins))
        return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    dim3 tb = d.grid_dim_2d, imgs = d.img_shape;
    void *args[] = {&tb, &imgs, &ids_sorted, &bins, &xys, &conics, &colors, &opac,
                    &final_Ts, &final_idx, &img, &bg};
    if (launch(K.raster_fwd, d.grid_dim_2d, d.block_dim_2d, s, args)) return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    HCHECK(cudaFreeAsync(ids_sorted, s));
    HCHECK(cudaFreeAsync(bins, s));
    HCHECK(cudaStreamSynchronize(s));
    return 0;
}

// lib/ops.cu:172-235 and 493-605
int ref_xla_rasterize_bwd(cudaStream_t s, void **b, const char *opaque, size_t len) {
    RefDescriptor d;
    if (unpack(opaque, len, &d)) return 1;
    const float3 *colors = (const float3 *)b[0];
    const float *opac = (const float *)b[1];
    const float3 *bg = (const float3 *)b[2];
    const float2 *xys = (const float2 *)b[3];
    const float *depths = (const float *)b[4];
    const int *radii = (const int *)b[5];
    const float3 *conics = (const float3 *)b[6];
    const int *cum = (const int *)b[7];
    const float *final_Ts = (const float *)b[8];
    const int *final_idx = (const int *)b[9];
    const float3 *v_img = (const float3 *)b[10];
    const float *v_alpha = (const float *)b[11];
    float3 *v_colors = (float3 *)b[12];
    float *v_opac = (float *)b[13];
    float2 *v_xy = (float2 *)b[14];
    float2 *v_xy_abs = (float2 *)b[15];
    float3 *v_conic = (float3 *)b[16];
    int num_isect = 0;
    HCHECK(cudaMemcpyAsync(&num_isect, cum + d.num_points - 1, sizeof(int),
                           cudaMemcpyDeviceToHost, s));
    size_t n = d.num_points;
    HCHECK(cudaMemsetAsync(v_xy, 0, n * sizeof(float2), s));
    HCHECK(cudaMemsetAsync(v_xy_abs, 0, n * sizeof(float2), s));
    HCHECK(cudaMemsetAsync(v_conic, 0, n * sizeof(float3), s));
    HCHECK(cudaMemsetAsync(v_colors, 0, n * sizeof(float3), s));
    HCHECK(cudaMemsetAsync(v_opac, 0, n * sizeof(float), s));
    int32_t *ids_sorted = nullptr;
    int2 *bins = nullptr;
    size_t ntiles = (size_t)d.grid_dim_2d.x * d.grid_dim_2d.y;
    HCHECK(cudaMallocAsync((void **)&ids_sorted, sizeof(int32_t) * (size_t)num_isect, s));
    HCHECK(cudaMemsetAsync(ids_sorted, 0, sizeof(int32_t) * (size_t)num_isect, s));
    HCHECK(cudaMallocAsync((void **)&bins, sizeof(int2) * ntiles, s));
    HCHECK(cudaMemsetAsync(bins, 0, sizeof(int2) * ntiles, s));
    HCHECK(cudaStreamSynchronize(s));
    if (num_isect == 0) return 0;
    if (sort_and_bin(s, d, (unsigned)num_isect, xys, depths, radii, cum, ids_sorted, bins))
        return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    dim3 tb = d.grid_dim_2d, imgs = d.img_shape;
    void *args[] = {&tb, &imgs, &ids_sorted, &bins, &xys, &conics, &colors, &opac, &bg,
                    &final_Ts, &final_idx, &v_img, &v_alpha, &v_xy, &v_xy_abs, &v_conic,
                    &v_colors, &v_opac};
    if (launch(K.raster_bwd, d.grid_dim_2d, d.block_dim_2d, s, args)) return 1;
    HCHECK(cudaGetLastError());
    HCHECK(cudaStreamSynchronize(s));
    HCHECK(cudaFreeAsync(ids_sorted, s));
    HCHECK(cudaFreeAsync(bins, s));
    HCHECK(cudaStreamSynchronize(s));
    return 0;
}

// Intermediates of lib/ops.cu:645-793 into caller buffers (keys_unsorted,
// ids_unsorted, keys_sorted, ids_sorted: `count` entries; bins: n_tiles int2,
// zeroed here as lib/ops.cu:482-488 does).
int ref_stage_sort_and_bin(cudaStream_t s, const char *opaque, size_t len, unsigned count,
                           const float2 *xys, const float *depths, const int *radii,
                           const int *cum, int64_t *keys_unsorted, int32_t *ids_unsorted,
                           int64_t *keys_sorted, int32_t *ids_sorted, int2 *bins) {
    RefDescriptor d;
    if (unpack(opaque, len, &d)) return 1;
    size_t ntiles = (size_t)d.grid_dim_2d.x * d.grid_dim_2d.y;
    HCHECK(cudaMemsetAsync(bins, 0, sizeof(int2) * ntiles, s));
    if (count == 0) return 0;
    if (map_isect(s, d, xys, depths, radii, cum, keys_unsorted, ids_unsorted)) return 1;
    if (sort_pairs(s, count, keys_unsorted, keys_sorted, ids_unsorted, ids_sorted,
                   end_bit_for(d)))
        return 1;
    if (bin_edges(s, d, count, keys_sorted, bins)) return 1;
    HCHECK(cudaStreamSynchronize(s));
    return 0;
}

}  // extern "C"
