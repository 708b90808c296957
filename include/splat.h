/*
 * splat.h -- C ABI of libsplat, the GB300 (sm_103a) Gaussian-splatting render
 * path that stands in for jaxsplat's native module.
 *
 * Two families of entry points:
 *
 *  1. splat_xla_*: the reference's XLA custom-call targets, with the same
 *     signature, buffer order and 80-byte opaque descriptor.  They replace
 *     the four PyCapsules that jaxsplat registers at import
 *     (lib/ffi.cu:4-13 registrations(), lib/ops.h:45-92):
 *         void fn(cudaStream_t, void **buffers, const char *opaque, size_t len)
 *     Like the reference they read the intersection count back to the host
 *     and take their temporaries from the stream-ordered allocator
 *     (cudaMallocAsync); unlike it they never synchronise the stream
 *     otherwise, never throw, and record failures for splat_last_error().
 *
 *  2. splat_*: typed entry points with plain pointers, sizes, an explicit
 *     stream, caller-provided workspace (size from the *_workspace_size
 *     query, 256-byte aligned: it holds words updated by 64-bit atomics;
 *     a misaligned one is refused with SPLAT_ERR_INVALID_ARG) and an int
 *     status.  tile_bins must be 8-byte aligned (read and written as int2)
 *     and packed 16-byte aligned (float4 records).  No allocation, no host synchronisation
 *     (except splat_read_counts, which exists to read the count).
 *
 * All arrays are row-major, C-contiguous, fp32 unless marked, with the
 * reference's shapes (jaxsplat/_project/abstract.py:7-77,
 * jaxsplat/_rasterize/abstract.py:7-85).  N = num_points, I = number of
 * tile/Gaussian intersections, T = tiles_x * tiles_y with
 * tiles_x = ceil(W / block_width), tiles_y = ceil(H / block_width).
 */
#ifndef SPLAT_H_
#define SPLAT_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SPLAT_API __attribute__((visibility("default")))
#else
#define SPLAT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *splat_stream_t; /* == cudaStream_t */

/* Status codes returned by every typed entry point. */
enum {
    SPLAT_OK = 0,
    SPLAT_ERR_INVALID_ARG = 1, /* bad size, shape, pointer or block width */
    SPLAT_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
    SPLAT_ERR_WORKSPACE = 3,   /* workspace smaller than *_workspace_size() */
    SPLAT_ERR_OVERFLOW = 4,    /* intersection count exceeds the supported range */
    SPLAT_ERR_DEVICE = 5       /* a device-side check fired (see splat_device_status_string) */
};

/*
 * Render parameters: the fields of ops::Descriptor (lib/ops.h:9-22) that
 * carry meaning, plus two controls of this library.
 *   block_width   tile side in pixels, 2..16 (the reference's limit:
 *                 block_width^2 <= MAX_GRID_DIM = 256, lib/common.h:9)
 *   device_status optional device pointer to one uint32 that kernels OR
 *                 failure bits into (NULL: checks still skip bad writes,
 *                 nothing is recorded)
 *   spin_limit    polls before a decoupled look-back wait gives up
 *                 (0 = default)
 */
typedef struct splat_params {
    uint32_t num_points;
    uint32_t img_height;
    uint32_t img_width;
    float fx, fy, cx, cy;
    float glob_scale;
    float clip_thresh;
    uint32_t block_width;
    uint32_t *device_status;
    uint32_t spin_limit;
} splat_params;

/* Thread-local message for the last failure in this thread. */
SPLAT_API const char *splat_last_error(void);
SPLAT_API const char *splat_status_string(int status);
/* Text for the bits of a device status word. */
SPLAT_API const char *splat_device_status_string(uint32_t bits);
SPLAT_API int splat_version(void);

/* ---------------------------------------------------------------------- */
/* Projection forward.  Replaces ops::project::fwd::xla (lib/ops.cu:12-61):
 * project_gaussians_fwd (lib/kernels/forward.cu:13-131) fused with the int32
 * inclusive scan of num_tiles_hit (lib/ops.cu:607-643) in one single-pass
 * kernel.  Every output element is written (zeros where the reference's
 * memsets leave zeros).
 *   means3d (N,3) scales (N,3) quats (N,4, w-x-y-z) viewmat (4,4)
 *   -> cov3d (N,6) xys (N,2) depths (N,1) radii (N,1) int32 conics (N,3)
 *      compensation (N,1) num_tiles_hit (N,1) int32 cum_tiles_hit (N,1) int32
 * total_out (optional, device int64): I as a 64-bit count.  cum_tiles_hit
 * may be NULL when total_out is given: then only the total is produced
 * (no scan). */
SPLAT_API size_t splat_project_fwd_workspace_size(const splat_params *p);
SPLAT_API int splat_project_fwd(const splat_params *p, const float *means3d, const float *scales,
                      const float *quats, const float *viewmat, float *cov3d, float *xys,
                      float *depths, int32_t *radii, float *conics, float *compensation,
                      int32_t *num_tiles_hit, int32_t *cum_tiles_hit, int64_t *total_out,
                      void *workspace, size_t workspace_bytes, splat_stream_t stream);

/* splat_project_fwd that also writes the rasterizers' packed records
 * (splat_pack_splats' output, bit-identical) from each Gaussian's projection
 * and its colour and opacity, so that no separate packing pass runs.  No
 * reference counterpart (the reference has no packing pass).  Same workspace.
 *   colors (N,3) opacities (N,1) -> packed (N,12), 16-byte aligned
 * cum_tiles_hit may be NULL here: the projection then only adds up the
 * intersection count into total_out (one atomic per block) instead of
 * scanning the tile counts. */
SPLAT_API int splat_project_fwd_packed(const splat_params *p, const float *means3d,
                                       const float *scales, const float *quats,
                                       const float *viewmat, const float *colors,
                                       const float *opacities, float *cov3d, float *xys,
                                       float *depths, int32_t *radii, float *conics,
                                       float *compensation, int32_t *num_tiles_hit,
                                       int32_t *cum_tiles_hit, int64_t *total_out,
                                       float *packed, void *workspace, size_t workspace_bytes,
                                       splat_stream_t stream);

/* Blocking read of the intersection count and, when status_dev is not NULL,
 * of the device status word (which is then cleared).  Replaces the D2H read
 * in lib/ops.cu:424-432.  total_dev: the int64 written by splat_project_fwd;
 * when NULL, cum_tiles_hit[N-1] is read instead. */
SPLAT_API int splat_read_counts(const splat_params *p, const int32_t *cum_tiles_hit,
                      const int64_t *total_dev, uint32_t *status_dev, int64_t *num_intersects,
                      uint32_t *status_out, splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Sort and bin.  Replaces ops::sort_and_bin (lib/ops.cu:645-793): the order
 * of a stable LSD radix sort of the 64-bit tile|depth keys of the reference's
 * emission (lib/kernels/forward.cu:135-179) over bits [0, 32+msb) (CUB
 * SortPairs at lib/ops.cu:728-757), and the tile bin edges
 * (lib/kernels/forward.cu:184-208).  Produced here by an in-house onesweep
 * radix sort of the Gaussians by depth, emission in depth order and a stable
 * radix sort by tile id.
 *   -> gaussian_ids_sorted (I,) int32, tile_bins (T,2) int32 (empty tiles (0,0))
 *   isect_ids / gaussian_ids (optional, both or neither): the reference's
 *     unsorted emission (needs cum_tiles_hit)
 *   isect_ids_sorted (optional): the sorted 64-bit keys
 * Counts: with count_dev == NULL, num_intersects is the exact count I.  With
 * count_dev (a device int64, e.g. splat_project_fwd's total_out) the count is
 * read on the device, num_intersects is the capacity the buffers and the
 * workspace were sized for, and nothing is read back to the host (the call is
 * CUDA-graph capturable); a count above the capacity sets the device status
 * bit "capacity-exceeded" and leaves the outputs unusable. */
SPLAT_API size_t splat_sort_workspace_size(const splat_params *p, int64_t num_intersects);
SPLAT_API int splat_sort_and_bin(const splat_params *p, int64_t num_intersects,
                                 const int64_t *count_dev, const float *xys,
                                 const float *depths, const int32_t *radii,
                                 const int32_t *cum_tiles_hit, int32_t *gaussian_ids_sorted,
                                 int32_t *tile_bins, int64_t *isect_ids, int32_t *gaussian_ids,
                                 int64_t *isect_ids_sorted, void *workspace,
                                 size_t workspace_bytes, splat_stream_t stream);

/* Pack the rasterizer's per-Gaussian inputs into one record each: (N,12)
 * floats, 16-byte aligned (x, y, conic a, b | conic c, opacity, r, g |
 * b, hx, hy, 0), where (hx, hy) bound the pixels at which the Gaussian can
 * pass the reference's alpha >= 1/255 test (a conservative box used only to
 * skip work that test would reject).  Inputs are the reference's rasterize
 * operands (jaxsplat/_rasterize/abstract.py:7-24):
 *   xys (N,2) conics (N,3) colors (N,3) opacities (N,1) -> packed (N,12) */
SPLAT_API int splat_pack_splats(const splat_params *p, const float *xys, const float *conics,
                                const float *colors, const float *opacities, float *packed,
                                splat_stream_t stream);

/* Rasterize forward over a sorted list.  Replaces the rasterize_fwd launch of
 * ops::rasterize::fwd::xla (lib/ops.cu:144-160, kernel
 * lib/kernels/forward.cu:339-462), including the empty-list path
 * (lib/ops.cu:119-127: image = background, final_Ts = final_idx = 0).
 * num_intersects / count_dev as for splat_sort_and_bin.
 *   packed (N,12) from splat_pack_splats, background (3,)
 *   -> final_Ts (H,W,1) final_idx (H,W,1) int32 out_img (H,W,3)
 *   blend_out (optional, block_width 16; ignored for other widths): one
 *     byte per sorted-list slot (num_intersects, or the capacity with
 *     count_dev), bit w set when some pixel of the tile's warp w (the 8x8
 *     pixel block at ((w & 1) * 8, (w >> 1) * 8)) passed that entry's alpha
 *     test.  Written for the entries up to the tile's largest final_idx;
 *     pass it to splat_rasterize_bwd, which then walks only those entries
 *     (no counterpart in the reference; NULL: not recorded). */
SPLAT_API int splat_rasterize_fwd(const splat_params *p, int64_t num_intersects,
                                  const int64_t *count_dev,
                                  const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                                  const float *packed, const float *background, float *final_Ts,
                                  int32_t *final_idx, float *out_img, uint8_t *blend_out,
                                  splat_stream_t stream);

/* splat_rasterize_fwd with the L2 loss of splat_l2_loss fused into its
 * epilogue (each pixel's colour is still in registers): additionally
 *   target (H,W,3) -> v_img (H,W,3) = 2 (img - target) / (3 H W), bit-identical
 *   to splat_l2_loss's, and loss_out[0] = mean((img - target)^2) (overwritten;
 *   summed per tile, so its last bits depend on the order of the tiles' adds,
 *   as splat_l2_loss's do on its blocks'). */
SPLAT_API int splat_rasterize_fwd_l2(const splat_params *p, int64_t num_intersects,
                                     const int64_t *count_dev,
                                     const int32_t *gaussian_ids_sorted,
                                     const int32_t *tile_bins, const float *packed,
                                     const float *background, const float *target,
                                     float *final_Ts, int32_t *final_idx, float *out_img,
                                     float *v_img, float *loss_out, uint8_t *blend_out,
                                     splat_stream_t stream);

/* Rasterize backward over the same sorted list (no re-sort).  Replaces the
 * rasterize_bwd launch of ops::rasterize::bwd::xla (lib/ops.cu:203-225,
 * kernel lib/kernels/backward.cu:153-343).  Outputs are overwritten.
 *   v_img (H,W,3) v_img_alpha (H,W,1)
 *   -> v_colors (N,3) v_opacity (N,1) v_xy (N,2) v_conic (N,3)
 *      v_xy_abs (N,2) optional: NULL skips the sum of |v_xy| that the
 *      reference computes and jaxsplat discards.
 *   blend (optional, block_width 16): the forward's blend_out over the same
 *     list; the backward then stages and walks only the entries some pixel
 *     of each warp passed (same results; NULL: every entry whose culling
 *     box meets the warp's pixels). */
SPLAT_API int splat_rasterize_bwd(const splat_params *p, int64_t num_intersects,
                                  const int64_t *count_dev,
                                  const int32_t *gaussian_ids_sorted, const int32_t *tile_bins,
                                  const float *packed, const float *background,
                                  const float *final_Ts, const int32_t *final_idx,
                                  const float *v_img, const float *v_img_alpha, float *v_colors,
                                  float *v_opacity, float *v_xy, float *v_xy_abs, float *v_conic,
                                  const uint8_t *blend, splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Projection backward.  Replaces ops::project::bwd::xla (lib/ops.cu:63-105,
 * kernel lib/kernels/backward.cu:345-418).  Outputs are overwritten.
 *   -> v_mean3d (N,3) v_scale (N,3) v_quat (N,4) v_cov2d (N,3) v_cov3d (N,6)
 * v_cov2d and v_cov3d (intermediate cotangents) may be NULL: not written. */
SPLAT_API int splat_project_bwd(const splat_params *p, const float *means3d, const float *scales,
                      const float *quats, const float *viewmat, const float *cov3d,
                      const int32_t *radii, const float *conics, const float *compensation,
                      const float *v_xy, const float *v_depth, const float *v_conic,
                      const float *v_compensation, float *v_mean3d, float *v_scale,
                      float *v_quat, float *v_cov2d, float *v_cov3d, splat_stream_t stream);

/* Work counts of one forward+backward over a sorted list, for a compute
 * roofline (diagnostic, no reference counterpart; one block per tile, not
 * on the step path).  Same list arguments as splat_rasterize_fwd plus the
 * forward's final_idx.  counts (device, 4 x uint64, overwritten):
 *   [0] pixel-Gaussian pairs the reference's forward evaluates (per pixel,
 *       list entries up to and including the saturating one,
 *       lib/kernels/forward.cu:380-455);
 *   [1] pairs its backward evaluates (entries up to final_idx,
 *       lib/kernels/backward.cu:240-262);
 *   [2] of those, the contributing pairs (sigma >= 0, alpha >= 1/255);
 *   [3] (tile, Gaussian) pairs with a contributing pixel (the granularity of
 *       the backward's gradient atomics, lib/kernels/backward.cu:314-340). */
SPLAT_API int splat_count_pairs(const splat_params *p, int64_t num_intersects,
                                const int64_t *count_dev, const int32_t *gaussian_ids_sorted,
                                const int32_t *tile_bins, const float *packed,
                                const int32_t *final_idx, uint64_t *counts,
                                splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Mean squared error against a target and its cotangent:
 * loss_out[0] = mean((img - target)^2), v_img = 2 (img - target) / count.
 * loss_out is overwritten.  (The loss of the reference's fitting example,
 * examples/single_image.py:26-29, used by the benchmark step.) */
SPLAT_API int splat_l2_loss(const float *img, const float *target, int64_t count, float *loss_out,
                  float *v_img, splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Fitting loop of examples/single_image.py:10-69 (quats normalised, colors
 * and opacities through a sigmoid, optax.adam(lr) on the raw parameters).
 * splat_fit_transform maps raw -> rendered parameters:
 *   quats (N,4) = quats_raw / |quats_raw|, colors (N,3) = sigmoid(colors_raw),
 *   opac (N,1) = sigmoid(opac_raw).
 * splat_fit_adam increments the device step counter *step_dev, then applies
 * the maps' chain rule to the render gradients (with respect to means,
 * scales and the mapped quats, colors, opacities) and one Adam update
 * (b1 0.9, b2 0.999, eps 1e-8) to the 14 raw parameters of every Gaussian;
 * m and v are (N,14) moment buffers (means 3, scales 3, quats 4, colors 3,
 * opacity 1), zero before the first step. */
SPLAT_API int splat_fit_transform(int n, const float *quats_raw, const float *colors_raw,
                                  const float *opac_raw, float *quats, float *colors,
                                  float *opac, splat_stream_t stream);
SPLAT_API int splat_fit_adam(int n, float lr, int *step_dev, float *means, float *scales,
                             float *quats_raw, float *colors_raw, float *opac_raw, float *m,
                             float *v, const float *g_means, const float *g_scales,
                             const float *g_quats, const float *g_colors, const float *g_opac,
                             const float *quats, const float *colors, const float *opac,
                             splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Legacy XLA custom-call targets (drop-in for lib/ffi.cu:4-13).  Buffers in
 * the order of jaxsplat/_{project,rasterize}/lowering.py; opaque is the
 * 80-byte descriptor of splat_xla_make_descriptor (lib/ffi.cu:15-52). */
SPLAT_API void splat_xla_project_fwd(splat_stream_t stream, void **buffers, const char *opaque,
                           size_t opaque_len);
SPLAT_API void splat_xla_project_bwd(splat_stream_t stream, void **buffers, const char *opaque,
                           size_t opaque_len);
SPLAT_API void splat_xla_rasterize_fwd(splat_stream_t stream, void **buffers, const char *opaque,
                             size_t opaque_len);
SPLAT_API void splat_xla_rasterize_bwd(splat_stream_t stream, void **buffers, const char *opaque,
                             size_t opaque_len);
/* img_shape is (H, W) as in jaxsplat; writes 80 bytes to out. */
SPLAT_API int splat_xla_make_descriptor(uint32_t num_points, uint32_t img_h, uint32_t img_w, float fx,
                              float fy, float cx, float cy, float glob_scale, float clip_thresh,
                              uint32_t block_width, void *out, size_t out_len);

/* ---------------------------------------------------------------------- */
/* Projection forward without a workspace (no counterpart in the reference).
 * For callers that cannot allocate device memory -- e.g. a plugin inside a
 * host application that owns and pools all device memory, or another
 * runtime's handler where cudaMalloc would synchronise or is not allowed.
 * Same inputs, outputs and results as splat_project_fwd; the scan's scratch
 * is a fixed device array inside the library (about 0.5 MB per GPU that
 * loads it, held until exit).
 *   - at most 16,777,216 Gaussians; larger inputs fail with
 *     SPLAT_ERR_INVALID_ARG before any GPU work;
 *   - uses the calling thread's current CUDA context: the array's device
 *     address belongs to that context, so the first call in each context
 *     (each device's primary context, again after cudaDeviceReset, and any
 *     context the host creates itself) looks the address up and caches it
 *     under the context's ID -- make that first call before any stream
 *     capture; a stream of another context fails with
 *     SPLAT_ERR_INVALID_ARG before any GPU work;
 *   - all calls on a device share the array: calls that overlap on the GPU
 *     race and must be ordered by the caller; each call clears the part it
 *     uses, so back-to-back calls are fine;
 *   - allocates nothing (no cudaMalloc/cudaFree, no allocator calls). */
SPLAT_API int splat_project_fwd_noalloc(const splat_params *p, const float *means3d,
                                        const float *scales, const float *quats,
                                        const float *viewmat, float *cov3d, float *xys,
                                        float *depths, int32_t *radii, float *conics,
                                        float *compensation, int32_t *num_tiles_hit,
                                        int32_t *cum_tiles_hit, int64_t *total_out,
                                        splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Batched render: many views of several scenes (uneven Gaussian counts and
 * image sizes) in one pass of each kernel.  No counterpart in the reference,
 * which renders one view per call (jaxsplat/__init__.py:6-70); every view's
 * image, final_Ts and gradients equal those of that view rendered alone
 * through the single-view entry points, and its final_idx too, shifted by
 * the number of intersections of the views before it (final_idx indexes the
 * batch's sorted list).  A view with no intersection at all keeps
 * final_Ts = 1 (the single-view call's empty-list path writes 0).
 *
 * Scenes are concatenated: scene s owns Gaussians [scene_base[s],
 * scene_base[s] + scene_points[s]) of the scene arrays (means3d (G,3),
 * scales (G,3), quats (G,4), colors (G,3), opacities (G,1)).  An "entry" is
 * one (view, Gaussian) pair; view v's entries start at a multiple of 256 and
 * the per-entry arrays (cov3d, xys, depths, radii, conics, compensation,
 * packed records, v_xy, v_conic) have num_entries rows, padding rows
 * included (written as culled Gaussians).  Tiles and pixels are numbered
 * view after view: view v's tile (tx, ty) is tile_base + ty*tiles_x + tx and
 * its pixel (y, x) is pixel_base + y*width + x of the pixel buffers (img
 * (P,3), final_Ts (P,1), final_idx (P,1), target, v_img, v_img_alpha).
 *
 * Fill each view's first block of fields, call splat_batch_layout on the
 * host array (it fills the derived fields and the totals), copy the array to
 * the device and point splat_batch::views at it. */
typedef struct splat_view {
    float viewmat[16];   /* row-major world -> camera */
    float fx, fy, cx, cy;
    float background[3];
    uint32_t scene;
    uint32_t img_height, img_width;
    /* derived by splat_batch_layout */
    uint32_t tiles_x, tiles_y;
    uint32_t gauss_base;  /* first Gaussian of the view's scene */
    uint32_t num_points;  /* the scene's Gaussian count */
    uint32_t entry_base;  /* first entry of the view (multiple of 256) */
    uint32_t tile_base;   /* first tile of the view */
    uint64_t pixel_base;  /* first pixel of the view */
} splat_view;

typedef struct splat_batch {
    uint32_t num_scenes, num_views;
    float glob_scale, clip_thresh;
    uint32_t block_width;          /* 2..16, shared by all views */
    uint32_t *device_status;       /* as in splat_params */
    uint32_t spin_limit;
    const splat_view *views;       /* device array of num_views */
    /* totals, derived by splat_batch_layout */
    uint64_t num_points;           /* Gaussians over all scenes */
    uint64_t num_entries, num_tiles, num_pixels;
} splat_batch;

/* Host: fills the derived fields of views[0..num_views) and b's totals from
 * scene_points[0..num_scenes) (the scenes' Gaussian counts; scene s starts at
 * the sum of the counts before it).  SPLAT_ERR_OVERFLOW when the scenes hold
 * more than 2^31 - 1 Gaussians in total or the views more than 2^31 - 1
 * entries or tiles (Gaussian ids, entries and tiles are int32 on the device). */
SPLAT_API int splat_batch_layout(splat_batch *b, splat_view *views, const uint32_t *scene_points);

/* Projection forward of every entry (forward.cu:13-131 per view; tile counts
 * are not kept).  total_dev (device int64) receives the number of
 * intersections over all views; it is overwritten. */
SPLAT_API int splat_batch_project_fwd(const splat_batch *b, const float *means3d,
                                      const float *scales, const float *quats, float *cov3d,
                                      float *xys, float *depths, int32_t *radii, float *conics,
                                      float *compensation, int64_t *total_dev,
                                      splat_stream_t stream);

/* splat_batch_project_fwd that also writes every entry's packed record
 * (splat_batch_pack's output, bit-identical), so that no packing pass runs.
 *   colors (G,3) opacities (G,1) -> packed (E,12), 16-byte aligned */
SPLAT_API int splat_batch_project_fwd_packed(const splat_batch *b, const float *means3d,
                                             const float *scales, const float *quats,
                                             const float *colors, const float *opacities,
                                             float *cov3d, float *xys, float *depths,
                                             int32_t *radii, float *conics, float *compensation,
                                             int64_t *total_dev, float *packed,
                                             splat_stream_t stream);

/* Sort and bin over all views, plus the order in which the rasterizers'
 * persistent blocks take tiles (longest tile list first).  capacity and
 * count_dev as for splat_sort_and_bin with a device count.
 *   -> gaussian_ids_sorted (capacity,) int32 entry ids, tile_bins (num_tiles,2),
 *      tile_order (num_tiles,) int32 */
SPLAT_API size_t splat_batch_sort_workspace_size(const splat_batch *b, int64_t capacity);
SPLAT_API int splat_batch_sort_and_bin(const splat_batch *b, int64_t capacity,
                                       const int64_t *count_dev, const float *xys,
                                       const float *depths, const int32_t *radii,
                                       int32_t *gaussian_ids_sorted, int32_t *tile_bins,
                                       int32_t *tile_order, void *workspace,
                                       size_t workspace_bytes, splat_stream_t stream);

/* Packed records of every entry (splat_pack_splats, with the colors and
 * opacities of the entry's scene Gaussian). */
SPLAT_API int splat_batch_pack(const splat_batch *b, const float *xys, const float *conics,
                               const float *colors, const float *opacities, float *packed,
                               splat_stream_t stream);

/* Rasterize forward / backward over all views with persistent blocks that
 * take `chunk` tiles at a time from tile_order (1..64).  The backward
 * overwrites v_colors (G,3) and v_opacity (G,1) (summed over the views of
 * each scene) and v_xy (E,2), v_conic (E,3) (per entry). */
SPLAT_API int splat_batch_rasterize_fwd(const splat_batch *b, int64_t capacity,
                                        const int64_t *count_dev,
                                        const int32_t *gaussian_ids_sorted,
                                        const int32_t *tile_bins, const int32_t *tile_order,
                                        const float *packed, float *final_Ts, int32_t *final_idx,
                                        float *out_img, uint32_t chunk, int32_t *work_counter,
                                        splat_stream_t stream);
SPLAT_API int splat_batch_rasterize_bwd(const splat_batch *b, int64_t capacity,
                                        const int64_t *count_dev,
                                        const int32_t *gaussian_ids_sorted,
                                        const int32_t *tile_bins, const int32_t *tile_order,
                                        const float *packed, const float *final_Ts,
                                        const int32_t *final_idx, const float *v_img,
                                        const float *v_img_alpha, float *v_colors,
                                        float *v_opacity, float *v_xy, float *v_conic,
                                        uint32_t chunk, int32_t *work_counter,
                                        splat_stream_t stream);

/* splat_batch_rasterize_fwd with splat_batch_l2_loss fused into its epilogue
 * (v_img bit-identical; loss_out summed per tile). */
SPLAT_API int splat_batch_rasterize_fwd_l2(const splat_batch *b, int64_t capacity,
                                           const int64_t *count_dev,
                                           const int32_t *gaussian_ids_sorted,
                                           const int32_t *tile_bins, const int32_t *tile_order,
                                           const float *packed, const float *target,
                                           float *final_Ts, int32_t *final_idx, float *out_img,
                                           float *v_img, float *loss_out, uint32_t chunk,
                                           int32_t *work_counter, splat_stream_t stream);

/* Sum over views of mean((img - target)^2) and its cotangent, per view
 * v_img = 2 (img - target) / (3 H W).  loss_out is overwritten. */
SPLAT_API int splat_batch_l2_loss(const splat_batch *b, const float *img, const float *target,
                                  float *loss_out, float *v_img, splat_stream_t stream);

/* Projection backward of every entry; the gradients of the scene arrays are
 * summed over the views of each scene.  Overwrites v_mean3d (G,3),
 * v_scale (G,3), v_quat (G,4). */
SPLAT_API int splat_batch_project_bwd(const splat_batch *b, const float *means3d,
                                      const float *scales, const float *quats,
                                      const float *cov3d, const int32_t *radii,
                                      const float *conics, const float *compensation,
                                      const float *v_xy, const float *v_conic, float *v_mean3d,
                                      float *v_scale, float *v_quat, splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* BF16 GEMM on the tensor cores (tcgen05 MMA, TMA operand loads, FP32
 * accumulation) for the warm-start network; no counterpart in the reference.
 *   C[M,N] fp32 row-major (ldc) = A[M,K] x B[N,K]^T (+ C when accumulate),
 *   A, B bf16 row-major (K contiguous; lda, ldb elements), 16-byte aligned,
 *   K, lda, ldb multiples of 8.  status_dev (optional device uint32) gets
 *   the look-back-timeout bit if a tensor-core wait runs out. */
SPLAT_API int splat_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int lda,
                              int ldb, int ldc, int accumulate, uint32_t *status_dev,
                              splat_stream_t stream);
/* The same product with either operand stored MN-major (transposed):
 *   a_mn = 0: A stored [M,K] (lda >= K);  a_mn = 1: A stored [K,M] (lda >= M),
 *   b_mn = 0: B stored [N,K] (ldb >= K);  b_mn = 1: B stored [K,N] (ldb >= N),
 *   C[M,N] = op(A) x op(B)^T (+ C when accumulate), op(A) = [M,K], op(B) = [N,K].
 * The weight gradient of a convolution (a reduction over pixel rows, both
 * operands MN-major) and its data gradient (the weights as stored, B
 * MN-major) need no transposed copies.  Operand rules as splat_gemm_bf16. */
SPLAT_API int splat_gemm_bf16_mn(const void *A, int a_mn, const void *B, int b_mn, float *C, int M,
                                 int N, int K, int lda, int ldb, int ldc, int accumulate,
                                 uint32_t *status_dev, splat_stream_t stream);
/* The same product with the bias, the activation and the output conversion
 * in the GEMM's epilogue (the fp32 product is never stored):
 *   y[M,N] = act(A[M,K] x B[N,K]^T + bias[N]), act = ReLU when relu != 0,
 *   written to exactly one of y16 (bf16) or y32 (fp32), row stride ldy.
 * K > 0; operand rules as splat_gemm_bf16. */
SPLAT_API int splat_gemm_bf16_bias_act(const void *A, const void *B, const float *bias, void *y16,
                                       float *y32, int M, int N, int K, int lda, int ldb, int ldy,
                                       int relu, uint32_t *status_dev, splat_stream_t stream);

/* Kernels around the GEMM for the warm-start network's 3x3 convolutions
 * (padding 1, stride 1 or 2) on NHWC bf16 activations; no counterpart in the
 * reference.
 *   im2col3x3: x (n,h,w,c) bf16 -> cols (n*ho*wo, kpad) bf16, column
 *     (ky*3 + kx)*c + ch, zeros past 9c (kpad >= 9c, a multiple of 8; cols
 *     16-byte aligned; n*h*w*c < 2^31)
 *   col2im3x3: dcols (n*ho*wo, kpad) fp32 -> dx (n,h,w,c) fp32 (overwritten)
 *   col2im_act3x3: the same gather through the previous layer's ReLU:
 *     dz (n,h,w,c) bf16 = dx * [y > 0] (y: that layer's bf16 output, NHWC),
 *     dbias (c) += dz's channel sums; c and kpad multiples of 4, c <= 4096,
 *     dcols 16-byte and y, dz 8-byte aligned
 *   bias_act:  y = act(acc + bias) (ReLU when relu != 0), rows x cols, to y
 *     (bf16) and/or y32 (fp32)
 *   act_grad:  dz = dy * [y > 0] (or dy) as bf16; dbias += column sums
 *   adam: w -= lr mhat / (sqrt(vhat) + 1e-8) (b1 0.9, b2 0.999, step >= 1),
 *     w16 (optional) = bf16(w) */
SPLAT_API int splat_nn_im2col3x3(const void *x, void *cols, int n, int h, int w, int c, int stride,
                                 int kpad, splat_stream_t stream);
SPLAT_API int splat_nn_col2im3x3(const float *dcols, float *dx, int n, int h, int w, int c,
                                 int stride, int kpad, splat_stream_t stream);
SPLAT_API int splat_nn_col2im_act3x3(const float *dcols, const void *y, void *dz, float *dbias,
                                     int n, int h, int w, int c, int stride, int kpad,
                                     splat_stream_t stream);
SPLAT_API int splat_nn_bias_act(const float *acc, const float *bias, void *y, float *y32,
                                int64_t rows, int cols, int relu, splat_stream_t stream);
SPLAT_API int splat_nn_act_grad(const float *dy, const void *y, void *dz, float *dbias,
                                int64_t rows, int cols, int relu, splat_stream_t stream);
SPLAT_API int splat_nn_adam(float *w, float *m, float *v, const float *g, void *w16, int64_t n,
                            float lr, int step, splat_stream_t stream);
/* Adam over up to 16 parameter arrays in one launch (each as splat_nn_adam;
 * w16 optional per array; an empty array may have NULL pointers). */
typedef struct splat_adam_seg {
    float *w, *m, *v;
    const float *g;
    void *w16;
    int64_t n;
} splat_adam_seg;
SPLAT_API int splat_nn_adam_multi(const splat_adam_seg *segs, int nseg, float lr, int step,
                                  splat_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Self-test of the bounded wait: one block waits on a flag that nothing
 * sets, with `limit` polls, then records DEV_LOOKBACK_TIMEOUT in *status_dev
 * (device uint32) and returns.  Exists so the timeout path can be exercised
 * without hanging a GPU. */
SPLAT_API int splat_selftest_wait_timeout(uint32_t limit, uint32_t *status_dev, splat_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SPLAT_H_ */
