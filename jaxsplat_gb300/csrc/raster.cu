// raster.cu -- tile rasterizer, forward and backward, and the per-Gaussian
// packing pass that feeds them.
//
// One block per tile.  Per-pixel arithmetic is the reference's
// (forward.cu:339-462, backward.cu:153-343), evaluated in the same order so
// that final_idx and the image are bit-identical; what differs is how the
// work is organised:
//
//  * pack_kernel turns (xys, conics, colors, opacities) into one 48-byte
//    record per Gaussian, with a conservative box around the pixels where its
//    alpha can reach 1/255 (see below).  A staged batch entry is three
//    16-byte loads instead of five scattered ones.
//  * While staging a batch, each thread tests its Gaussian's box against the
//    pixel rectangle of every warp of the tile and stores a warp mask; each
//    warp then compacts the batch into the list of entries with its bit set
//    and walks only those.  The skipped ones are Gaussians that the
//    reference's per-pixel test (alpha < 1/255) rejects at every pixel of
//    the warp anyway.
//  * 16x16 tiles (raster_fwd16_kernel, raster_bwd16_kernel): 128 threads,
//    each warp an 8x8 pixel block, each lane two pixels of one column.  The
//    two pixels share dx, and their arithmetic runs as paired fp32
//    instructions (FFMA2/FMUL2/FADD2) that round each component exactly as
//    the scalar instruction would.  Other widths: one pixel per thread,
//    row-major (raster_fwd_kernel, raster_bwd_kernel).
//  * backward: the block starts at the largest final_idx of its pixels;
//    per-Gaussian sums are reduced across the warp with a transposed butterfly
//    (9 shuffles for 8 values) when many lanes contribute, or added per lane
//    when few do, and go to global memory with one atomic per field per
//    (warp, Gaussian).
#include <math_constants.h>

#include <algorithm>

#include "splat_internal.cuh"
#include "splat_math.cuh"

namespace splat {

constexpr int kMaxTile = 256;  // bw * bw <= 256
constexpr int kMaxWarps = kMaxTile / 32;

// ---------------------------------------------------------------------------
// Packing: one 48-byte record per Gaussian (write_record in splat_math.cuh,
// with the record layout and the proof of its culling box).

struct PackArgs {
    int n;
    const float *xys, *conics, *colors, *opac;
    float4 *rec;
};

// Record of entry i whose colour and opacity are those of Gaussian gc; the
// last word carries gc (as int bits) for the batched backward.
__device__ __forceinline__ void pack_record(const PackArgs &a, size_t i, size_t gc, float tag) {
    const float2 xy = *reinterpret_cast<const float2 *>(a.xys + 2 * i);
    const float3 conic = make_float3(a.conics[3 * i], a.conics[3 * i + 1], a.conics[3 * i + 2]);
    const float3 rgb = make_float3(a.colors[3 * gc], a.colors[3 * gc + 1], a.colors[3 * gc + 2]);
    write_record(a.rec + 3 * i, xy, conic, a.opac[gc], rgb, tag);
}

__global__ void __launch_bounds__(256) pack_kernel(PackArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    pack_record(a, (size_t)i, (size_t)i, 0.f);
}

// Batched views: entry i of view v packs Gaussian gauss_base + (i -
// entry_base) of its scene; padding entries (past the scene's count) get a
// record that no pixel passes.
__global__ void __launch_bounds__(256) pack_batch_kernel(PackArgs a, const splat_view *views,
                                                         int nviews) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const splat_view &v = views[view_by_entry(views, nviews, (uint32_t)i)];
    const uint32_t k = (uint32_t)i - v.entry_base;
    if (k < v.num_points) {
        const uint32_t gc = v.gauss_base + k;
        pack_record(a, (size_t)i, gc, __int_as_float((int)gc));
    } else {
        float4 *r = a.rec + 3 * (size_t)i;
        r[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        r[1] = make_float4(0.f, 0.f, 0.f, 0.f);
        r[2] = make_float4(0.f, -CUDART_INF_F, -CUDART_INF_F, __int_as_float((int)v.gauss_base));
    }
}

// ---------------------------------------------------------------------------
// Pixel layout and warp rectangles.

// Thread -> pixel of the tile for the one-pixel-per-thread kernels (tile
// widths other than 16): row-major.
__device__ __forceinline__ void pixel_of(int tr, int bw, int &tx, int &ty) {
    tx = tr % bw;
    ty = tr / bw;
}

// Bounding rectangle of the pixel centres of warp w (row-major pixels), in
// image coordinates (x_lo, x_hi, y_lo, y_hi).
__device__ __forceinline__ float4 warp_rect(int w, int bw, int bsize, float ox, float oy) {
    const int first = 32 * w, last = min(first + 31, bsize - 1);
    const int y0 = first / bw, y1 = last / bw;
    int x0 = 0, x1 = bw - 1;
    if (y0 == y1) {
        x0 = first % bw;
        x1 = last % bw;
    }
    return make_float4(ox + (float)x0 + 0.5f, ox + (float)x1 + 0.5f, oy + (float)y0 + 0.5f,
                       oy + (float)y1 + 0.5f);
}

// Bit w set unless the Gaussian of record (r0, r2) provably misses every
// pixel centre of warp w (they all lie outside its box).  NaN anywhere keeps
// the bit.
__device__ __forceinline__ unsigned warp_mask(float4 r0, float4 r2, const float4 *rects,
                                              int nwarps) {
    const float x = r0.x, y = r0.y, hx = r2.y, hy = r2.z;
    unsigned m = 0;
#pragma unroll
    for (int w = 0; w < kMaxWarps; ++w) {
        if (w >= nwarps) break;
        const float4 r = rects[w];
        const bool out = (x + hx < r.x) || (x - hx > r.y) || (y + hy < r.z) || (y - hy > r.w);
        if (!out) m |= 1u << w;
    }
    return m;
}

// Compacts, in order, the batch entries t in [t0, n) whose mask has this
// warp's bit into list[]; returns their number.  Warp-synchronous over the
// lanes in wmask.
__device__ __forceinline__ int warp_list(const unsigned *mask, int t0, int n, int warp, int lane,
                                         unsigned wmask, uint8_t *list) {
    int cnt = 0;
    const unsigned lt = (1u << lane) - 1u;
    const int lanes = __popc(wmask);  // a partial last warp has lanes 0 .. lanes-1
    for (int base = t0; base < n; base += lanes) {
        const int t = base + lane;
        const bool keep = t < n && ((mask[t] >> warp) & 1u);
        const unsigned bal = __ballot_sync(wmask, keep);
        if (keep) list[cnt + __popc(bal & lt)] = (uint8_t)t;
        cnt += __popc(bal);
    }
    __syncwarp(wmask);
    return cnt;
}

// ---------------------------------------------------------------------------
// Where a tile's pixels live.  Single-view launches take the tile from the
// block index; batched launches take it from a work list and the view table.

struct TileCtx {
    int tile;               // index into the tile bins
    unsigned ox, oy;        // pixel origin of the tile within its image
    unsigned width, height; // image size
    size_t pix_base;        // first pixel of the image in the pixel buffers
    float3 bg;
};

__device__ __forceinline__ TileCtx grid_tile(unsigned tiles_x, unsigned bw, unsigned width,
                                             unsigned height, const float *background) {
    TileCtx c;
    c.tile = (int)(blockIdx.y * tiles_x + blockIdx.x);
    c.ox = blockIdx.x * bw;
    c.oy = blockIdx.y * bw;
    c.width = width;
    c.height = height;
    c.pix_base = 0;
    c.bg = make_float3(background[0], background[1], background[2]);
    return c;
}

// ---------------------------------------------------------------------------
// Forward.

struct RasterFwdArgs {
    unsigned tiles_x, width, height, bw;
    int n;
    uint32_t *status;
    Count count;
    const int32_t *ids;
    const int2 *bins;
    const float4 *rec;
    const float *background;
    float *final_Ts;
    int32_t *final_idx;
    float *img;
    // kLoss: the L2 loss against `target` (same layout as img), as
    // splat_l2_loss computes it: v_img = 2 (img - target) / count, and the
    // tile's share of mean((img - target)^2) added to *loss.  Batched views:
    // count is the tile's view's 3 W H (splat_batch_l2_loss's per-view means,
    // summed), inv_count unused.
    const float *target;
    float *v_img, *loss;
    float inv_count;
    // Optional (16x16 tiles): one byte per sorted-list slot, bit w set when
    // some pixel of warp w passed that entry's alpha test (it blended the
    // entry, or saturated at it); the backward walks only those entries.
    // Written for every entry of each batch the tile processes (all entries
    // up to the tile's largest final_idx).
    uint8_t *blend;
};

// The L2 loss terms of one pixel (inside the image); returns its squared error.
__device__ __forceinline__ float pixel_l2(const RasterFwdArgs &a, size_t pix, float inv, float r,
                                          float g, float b) {
    const float v[3] = {r, g, b};
    float sq = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float d = v[k] - a.target[3 * pix + k];
        a.v_img[3 * pix + k] = 2.f * d * inv;
        sq += d * d;
    }
    return sq;
}

// Block sum of the squared errors, one atomic per tile.  Warp 0 sums the
// staged values (a block of fewer than 32 threads: thread 0 alone).
__device__ __forceinline__ void tile_l2_sum(const RasterFwdArgs &a, float sq, float inv,
                                            int bsize) {
    __shared__ float s_sq[kMaxTile];
    const int tr = threadIdx.x;
    s_sq[tr] = sq;
    __syncthreads();
    if (bsize >= 32) {
        if (tr < 32) {
            float t = 0.f;
            for (int k = tr; k < bsize; k += 32) t += s_sq[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (tr == 0) atomicAdd(a.loss, t * inv);
        }
    } else if (tr == 0) {
        float t = 0.f;
        for (int k = 0; k < bsize; ++k) t += s_sq[k];
        atomicAdd(a.loss, t * inv);
    }
}

template <bool kLoss = false, bool kViewLoss = false>
__device__ __forceinline__ void fwd_tile(const RasterFwdArgs &a, const TileCtx &c) {
    __shared__ float4 s_r0[kMaxTile];
    __shared__ float4 s_r1[kMaxTile];
    __shared__ float s_blue[kMaxTile];
    __shared__ unsigned s_mask[kMaxTile];
    __shared__ float4 s_rect[kMaxWarps];
    __shared__ uint8_t s_list[kMaxWarps][kMaxTile];
    const int tile = c.tile;
    const int tr = threadIdx.x;
    const int bsize = a.bw * a.bw;
    const int lane = tr & 31, warp = tr >> 5, nwarps = (bsize + 31) >> 5;
    const unsigned wmask = (warp == nwarps - 1 && (bsize & 31)) ? ((1u << (bsize & 31)) - 1u)
                                                                : 0xffffffffu;
    int tx, ty;
    pixel_of(tr, a.bw, tx, ty);
    const unsigned i = c.oy + ty;
    const unsigned j = c.ox + tx;
    const float px = (float)j + 0.5f;
    const float py = (float)i + 0.5f;
    const bool inside = i < c.height && j < c.width;
    const size_t pix = c.pix_base + (size_t)i * c.width + j;
    const float3 bg = c.bg;

    // the loss's 1 / count: the image's, or (batched views) the tile's view's,
    // formed as splat_batch_l2_loss forms it
    const float inv = kViewLoss ? 1.f / (3.f * (float)c.width * (float)c.height) : a.inv_count;
    if (a.count.get() == 0) {  // lib/ops.cu:119-127: background image, zero T and index
        float sq = 0.f;
        if (inside) {
            a.final_Ts[pix] = 0.f;
            a.final_idx[pix] = 0;
            a.img[3 * pix] = bg.x;
            a.img[3 * pix + 1] = bg.y;
            a.img[3 * pix + 2] = bg.z;
            if (kLoss) sq = pixel_l2(a, pix, inv, bg.x, bg.y, bg.z);
        }
        if (kLoss) tile_l2_sum(a, sq, inv, bsize);
        return;
    }
    if (tr < nwarps) s_rect[tr] = warp_rect(tr, a.bw, bsize, (float)c.ox, (float)c.oy);
    const int2 range = a.bins[tile];
    bool done = !inside;
    float T = 1.f;
    int cur_idx = 0;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    for (int start = range.x; start < range.y; start += bsize) {
        if (__syncthreads_count(done) >= bsize) break;  // also publishes s_rect
        const int idx = start + tr;
        if (idx < range.y) {
            const int g = a.ids[idx];
            if (g >= 0 && g < a.n) {
                const float4 r0 = a.rec[3 * (size_t)g];
                const float4 r1 = a.rec[3 * (size_t)g + 1];
                const float4 r2 = a.rec[3 * (size_t)g + 2];
                s_r0[tr] = r0;
                s_r1[tr] = r1;
                s_blue[tr] = r2.x;
                s_mask[tr] = warp_mask(r0, r2, s_rect, nwarps);
            } else {  // corrupt list entry: never contributes
                raise_status(a.status, DEV_BAD_ID);
                s_mask[tr] = 0u;
            }
        }
        __syncthreads();
        const int n = min(bsize, range.y - start);
        const int cnt = warp_list(s_mask, 0, n, warp, lane, wmask, s_list[warp]);
        // two entries per iteration: their loads and exponentials are
        // independent, the blending stays in list order
        int k = 0;
        for (; k + 1 < cnt && !done; k += 2) {
            const int t0 = s_list[warp][k], t1 = s_list[warp][k + 1];
            const float4 p0 = s_r0[t0], q0 = s_r1[t0];
            const float4 p1 = s_r0[t1], q1 = s_r1[t1];
            const float sg0 = falloff(p0.z, p0.w, q0.x, p0.x - px, p0.y - py);
            const float sg1 = falloff(p1.z, p1.w, q1.x, p1.x - px, p1.y - py);
            const float al0 = fminf(0.999f, q0.y * __expf(-sg0));
            const float al1 = fminf(0.999f, q1.y * __expf(-sg1));
            if (!(sg0 < 0.f || al0 < 1.f / 255.f)) {
                const float next_T = T * (1.f - al0);
                if (next_T <= 1e-4f) {
                    done = true;
                    break;
                }
                const float vis = al0 * T;
                acc.x = blend(acc.x, q0.z, vis);
                acc.y = blend(acc.y, q0.w, vis);
                acc.z = blend(acc.z, s_blue[t0], vis);
                T = next_T;
                cur_idx = start + t0;
            }
            if (!(sg1 < 0.f || al1 < 1.f / 255.f)) {
                const float next_T = T * (1.f - al1);
                if (next_T <= 1e-4f) {
                    done = true;
                    break;
                }
                const float vis = al1 * T;
                acc.x = blend(acc.x, q1.z, vis);
                acc.y = blend(acc.y, q1.w, vis);
                acc.z = blend(acc.z, s_blue[t1], vis);
                T = next_T;
                cur_idx = start + t1;
            }
        }
        if (k < cnt && !done) {
            const int t = s_list[warp][k];
            const float4 r0 = s_r0[t];
            const float4 r1 = s_r1[t];
            const float sigma = falloff(r0.z, r0.w, r1.x, r0.x - px, r0.y - py);
            const float alpha = fminf(0.999f, r1.y * __expf(-sigma));
            if (!(sigma < 0.f || alpha < 1.f / 255.f)) {
                const float next_T = T * (1.f - alpha);
                if (next_T <= 1e-4f) {
                    done = true;
                } else {
                    const float vis = alpha * T;
                    acc.x = blend(acc.x, r1.z, vis);
                    acc.y = blend(acc.y, r1.w, vis);
                    acc.z = blend(acc.z, s_blue[t], vis);
                    T = next_T;
                    cur_idx = start + t;
                }
            }
        }
    }
    float sq = 0.f;
    if (inside) {
        a.final_Ts[pix] = T;
        a.final_idx[pix] = cur_idx;
        const float r = blend(acc.x, T, bg.x), g = blend(acc.y, T, bg.y), b = blend(acc.z, T, bg.z);
        a.img[3 * pix] = r;
        a.img[3 * pix + 1] = g;
        a.img[3 * pix + 2] = b;
        if (kLoss) sq = pixel_l2(a, pix, inv, r, g, b);
    }
    if (kLoss) tile_l2_sum(a, sq, inv, bsize);
}

// Pixel centres of the 8x8 block of warp w in the two-pixels-per-thread
// 16x16 layout (x_lo, x_hi, y_lo, y_hi).
__device__ __forceinline__ float4 warp_rect16(int w, float ox, float oy) {
    const float x0 = (float)((w & 1) * 8), y0 = (float)((w >> 1) * 8);
    return make_float4(ox + x0 + 0.5f, ox + x0 + 7.5f, oy + y0 + 0.5f, oy + y0 + 7.5f);
}

// Paired fp32 arithmetic (sm_100+ FFMA2/FMUL2/FADD2): one instruction, two
// independent IEEE operations rounded to nearest.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float hsum(float2 a) { return a.x + a.y; }

// falloff() for one Gaussian at two pixels sharing dx (same roundings per
// component).
__device__ __forceinline__ float2 falloff2(float a, float b, float c, float dx, float2 dy) {
    const float2 cdy2 = mul2(mul2(f2(c), dy), dy);
    const float2 inner = fma2(f2(__fmul_rn(a, dx)), f2(dx), cdy2);
    return fma2(f2(__fmul_rn(b, dx)), dy, mul2(f2(0.5f), inner));
}

// ---------------------------------------------------------------------------
// Forward for 16x16 tiles: two pixels per thread, in the backward's layout.
// 128 threads; warp w owns the 8x8 pixel block at ((w & 1) * 8, (w >> 1) * 8),
// lane l the pixels (x, y) and (x, y + 4) with x = l & 7, y = l >> 3 inside
// it.  The two pixels share dx, and their falloff, alpha, transmittance and
// colour updates run as paired fp32 instructions (FFMA2/FMUL2/FADD2), each
// component rounded exactly as the scalar code rounds it, so the image,
// final_Ts and final_idx are those of the one-pixel-per-thread kernel bit for
// bit.  A warp walks its list while any of its pixels is unsaturated;
// saturated or non-passing pixels run the blend with alpha = 0, which leaves
// their state unchanged.

constexpr int kF16Threads = 128;
constexpr int kF16Warps = 4;
constexpr int kF16Batch = 256;

// The warps that passed each entry of a batch: byte w of word e is set by
// warp w (plain byte stores, one warp per byte), then packed to bits 0-3.
__device__ __forceinline__ uint8_t pack_blend_bytes(uint32_t x) {
    x &= 0x01010101u;
    return (uint8_t)((x | (x >> 7) | (x >> 14) | (x >> 21)) & 0xFu);
}

template <bool kLoss, bool kViewLoss, bool kBlend = false>
__device__ __forceinline__ void fwd16_tile(const RasterFwdArgs &a, const TileCtx &c) {
    __shared__ uint32_t s_blend[kBlend ? kF16Batch : 1];
    __shared__ float4 s_r0[kF16Batch];
    __shared__ float4 s_r1[kF16Batch];
    __shared__ float s_blue[kF16Batch];
    __shared__ unsigned s_mask[kF16Batch];
    __shared__ float4 s_rect[kF16Warps];
    __shared__ uint8_t s_list[kF16Warps][kF16Batch];
    const int tile = c.tile;
    const int tr = threadIdx.x, lane = tr & 31, warp = tr >> 5;
    const unsigned j = c.ox + ((warp & 1) << 3) + (lane & 7);
    const unsigned i0 = c.oy + ((warp >> 1) << 3) + (lane >> 3);
    const float px = (float)j + 0.5f;
    const bool in0 = i0 < c.height && j < c.width;
    const bool in1 = i0 + 4 < c.height && j < c.width;
    const size_t pix0 = c.pix_base + (size_t)i0 * c.width + j;
    const size_t pix1 = pix0 + 4 * (size_t)c.width;
    const float3 bg = c.bg;
    const float inv = kViewLoss ? 1.f / (3.f * (float)c.width * (float)c.height) : a.inv_count;

    if (a.count.get() == 0) {  // lib/ops.cu:119-127: background image, zero T and index
        float sq = 0.f;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!(q ? in1 : in0)) continue;
            const size_t pix = q ? pix1 : pix0;
            a.final_Ts[pix] = 0.f;
            a.final_idx[pix] = 0;
            a.img[3 * pix] = bg.x;
            a.img[3 * pix + 1] = bg.y;
            a.img[3 * pix + 2] = bg.z;
            if (kLoss) sq += pixel_l2(a, pix, inv, bg.x, bg.y, bg.z);
        }
        if (kLoss) tile_l2_sum(a, sq, inv, kF16Threads);
        return;
    }
    if (tr < kF16Warps) s_rect[tr] = warp_rect16(tr, (float)c.ox, (float)c.oy);
    const int2 range = a.bins[tile];
    const float2 neg_py = make_float2(-((float)i0 + 0.5f), -((float)(i0 + 4) + 0.5f));
    bool done0 = !in0, done1 = !in1;
    float2 T = make_float2(1.f, 1.f);
    float2 acc_r = make_float2(0.f, 0.f), acc_g = acc_r, acc_b = acc_r;
    int cur0 = 0, cur1 = 0;
    int prev_start = 0, prev_n = 0;  // the batch whose blend bytes are pending
    auto flush_blend = [&]() {
        for (int e = tr; e < prev_n; e += kF16Threads)
            a.blend[prev_start + e] = pack_blend_bytes(s_blend[e]);
    };
    for (int start = range.x; start < range.y; start += kF16Batch) {
        // also publishes s_rect, and orders the previous batch's walk before
        // its blend bytes are read
        const int all_done = __syncthreads_count(done0 && done1);
        if (kBlend) {
            flush_blend();
            prev_n = 0;
        }
        if (all_done >= kF16Threads) break;
        for (int e = tr; e < kF16Batch; e += kF16Threads) {
            const int idx = start + e;
            if (kBlend) s_blend[e] = 0u;
            if (idx < range.y) {
                const int g = a.ids[idx];
                if (g >= 0 && g < a.n) {
                    const float4 r0 = a.rec[3 * (size_t)g];
                    const float4 r1 = a.rec[3 * (size_t)g + 1];
                    const float4 r2 = a.rec[3 * (size_t)g + 2];
                    s_r0[e] = r0;
                    s_r1[e] = r1;
                    s_blue[e] = r2.x;
                    s_mask[e] = warp_mask(r0, r2, s_rect, kF16Warps);
                } else {  // corrupt list entry: never contributes
                    raise_status(a.status, DEV_BAD_ID);
                    s_mask[e] = 0u;
                }
            }
        }
        __syncthreads();
        const int n = min(kF16Batch, range.y - start);
        const int cnt = warp_list(s_mask, 0, n, warp, lane, 0xffffffffu, s_list[warp]);
        // Two list entries per iteration: both entries' falloffs and
        // exponentials are independent and go first, the blends follow in
        // list order (the arithmetic per entry is unchanged).
        // blend_entry: the blend of one entry whose falloff and opacity x
        // exponent are known; returns true when every pixel of the warp is
        // saturated.
        auto blend_entry = [&](int t, const float4 &r1, float2 sigma, float2 ov) -> bool {
            const float al0 = fminf(0.999f, ov.x), al1 = fminf(0.999f, ov.y);
            const bool pass0 = !done0 && !(sigma.x < 0.f || al0 < 1.f / 255.f);
            const bool pass1 = !done1 && !(sigma.y < 0.f || al1 < 1.f / 255.f);
            if (!__any_sync(0xffffffffu, pass0 || pass1))
                return __all_sync(0xffffffffu, done0 && done1);
            const float2 al = make_float2(pass0 ? al0 : 0.f, pass1 ? al1 : 0.f);
            const float2 next_T = mul2(T, fma2(al, f2(-1.f), f2(1.f)));  // T (1 - alpha)
            // a pixel whose next T would fall to 1e-4 stops before this
            // Gaussian (forward.cu:432-436)
            const bool stop0 = pass0 && next_T.x <= 1e-4f;
            const bool stop1 = pass1 && next_T.y <= 1e-4f;
            const bool bl0 = pass0 && !stop0, bl1 = pass1 && !stop1;
            // some pixel of this warp passed the entry's test: it blended
            // the entry, or stopped at it (the one entry past its final_idx
            // that the backward then walks for nothing)
            if (kBlend && lane == 0) reinterpret_cast<uint8_t *>(s_blend)[4 * t + warp] = 1;
            const float2 vis = mul2(make_float2(bl0 ? al0 : 0.f, bl1 ? al1 : 0.f), T);
            acc_r = fma2(f2(r1.z), vis, acc_r);
            acc_g = fma2(f2(r1.w), vis, acc_g);
            acc_b = fma2(f2(s_blue[t]), vis, acc_b);
            T = make_float2(bl0 ? next_T.x : T.x, bl1 ? next_T.y : T.y);
            if (bl0) cur0 = start + t;
            if (bl1) cur1 = start + t;
            done0 |= stop0;
            done1 |= stop1;
            return false;
        };
        auto eval = [&](const float4 &r0, const float4 &r1, float2 &sigma, float2 &ov) {
            const float dx = r0.x - px;
            const float2 dy = add2(f2(r0.y), neg_py);
            sigma = falloff2(r0.z, r0.w, r1.x, dx, dy);
            ov = mul2(f2(r1.y), make_float2(__expf(-sigma.x), __expf(-sigma.y)));
        };
        int k = 0;
        bool warp_done = false;
        for (; k + 1 < cnt; k += 2) {
            const int ta = s_list[warp][k], tb = s_list[warp][k + 1];
            const float4 r0a = s_r0[ta], r1a = s_r1[ta], r0b = s_r0[tb], r1b = s_r1[tb];
            float2 sa, oa, sb, ob;
            eval(r0a, r1a, sa, oa);
            eval(r0b, r1b, sb, ob);
            if ((warp_done = blend_entry(ta, r1a, sa, oa))) break;
            if ((warp_done = blend_entry(tb, r1b, sb, ob))) break;
        }
        if (!warp_done && k < cnt) {
            const int t = s_list[warp][k];
            const float4 r0 = s_r0[t], r1 = s_r1[t];
            float2 sg, o;
            eval(r0, r1, sg, o);
            blend_entry(t, r1, sg, o);
        }
        if (kBlend) {
            prev_start = start;
            prev_n = n;
        }
    }
    if (kBlend && prev_n) {
        __syncthreads();
        flush_blend();
    }
    float sq = 0.f;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        if (!(q ? in1 : in0)) continue;
        const size_t pix = q ? pix1 : pix0;
        const float Tq = q ? T.y : T.x;
        a.final_Ts[pix] = Tq;
        a.final_idx[pix] = q ? cur1 : cur0;
        const float r = blend(q ? acc_r.y : acc_r.x, Tq, bg.x);
        const float g = blend(q ? acc_g.y : acc_g.x, Tq, bg.y);
        const float b = blend(q ? acc_b.y : acc_b.x, Tq, bg.z);
        a.img[3 * pix] = r;
        a.img[3 * pix + 1] = g;
        a.img[3 * pix + 2] = b;
        if (kLoss) sq += pixel_l2(a, pix, inv, r, g, b);
    }
    if (kLoss) tile_l2_sum(a, sq, inv, kF16Threads);
}

template <bool kLoss, bool kBlend>
__global__ void __launch_bounds__(kF16Threads) raster_fwd16_kernel(RasterFwdArgs a) {
    fwd16_tile<kLoss, false, kBlend>(a, grid_tile(a.tiles_x, 16, a.width, a.height,
                                                  a.background));
}

template <bool kLoss>
__global__ void __launch_bounds__(kMaxTile) raster_fwd_kernel(RasterFwdArgs a) {
    fwd_tile<kLoss>(a, grid_tile(a.tiles_x, a.bw, a.width, a.height, a.background));
}

// ---------------------------------------------------------------------------
// Backward.

// Sums over the warp of 8 values, transposed, and of one more value `op`:
// on return lane L holds the warp total of value (L >> 2) & 7, and *op_total
// the total of op in every lane.  Each step exchanges half of what a lane
// holds with the lane 16, 8, then 4 apart (keeping the other half), then
// finishes with two full butterfly steps; op takes five butterfly steps.
// The adds of independent values issue as paired fp32 instructions (FADD2:
// each component rounded as the scalar add; every sum keeps its order).
// `lane` is the caller's lane index (the pixel layout decides it, not
// threadIdx.x).
__device__ __forceinline__ float warp_sum9_transposed(const float v[8], float op, int lane,
                                                      float *op_total) {
    const bool u16 = lane & 16, u8 = lane & 8, u4 = lane & 4;
    float2 b[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float s0 = u16 ? v[2 * k] : v[2 * k + 4], s1 = u16 ? v[2 * k + 1] : v[2 * k + 5];
        const float k0 = u16 ? v[2 * k + 4] : v[2 * k], k1 = u16 ? v[2 * k + 5] : v[2 * k + 1];
        b[k] = __fadd2_rn(make_float2(k0, k1), make_float2(__shfl_xor_sync(0xffffffffu, s0, 16),
                                                           __shfl_xor_sync(0xffffffffu, s1, 16)));
    }
    // b[0] = fields (0,1) or (4,5), b[1] = (2,3) or (6,7): step 2 keeps one pair
    const float2 sendp = u8 ? b[0] : b[1], keepp = u8 ? b[1] : b[0];
    const float2 c = __fadd2_rn(keepp, make_float2(__shfl_xor_sync(0xffffffffu, sendp.x, 8),
                                                   __shfl_xor_sync(0xffffffffu, sendp.y, 8)));
    const float send = u4 ? c.x : c.y;
    const float keep = u4 ? c.y : c.x;
    float o = op + __shfl_xor_sync(0xffffffffu, op, 16);
    o += __shfl_xor_sync(0xffffffffu, o, 8);
    o += __shfl_xor_sync(0xffffffffu, o, 4);
    float2 e = make_float2(keep + __shfl_xor_sync(0xffffffffu, send, 4), o);
    e = __fadd2_rn(e, make_float2(__shfl_xor_sync(0xffffffffu, e.x, 2),
                                  __shfl_xor_sync(0xffffffffu, e.y, 2)));
    e = __fadd2_rn(e, make_float2(__shfl_xor_sync(0xffffffffu, e.x, 1),
                                  __shfl_xor_sync(0xffffffffu, e.y, 1)));
    *op_total = e.y;
    return e.x;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Gradient fields of a (warp, Gaussian) pair.
enum { G_R, G_G, G_B, G_CA, G_CB, G_CC, G_X, G_Y, G_OP, G_AX, G_AY, G_FIELDS };

// With at most this many contributing lanes a warp's lanes add their own
// sums to the global gradients instead of reducing across the warp first
// (swept at 1920x1080: 12-14 fastest with the paired-add reduction, 16
// before it; 20 is 4 % slower).
constexpr int kFewLanes = 14;

struct RasterBwdArgs {
    unsigned tiles_x, width, height, bw;
    int n;
    uint32_t *status;
    Count count;
    const int32_t *ids;
    const int2 *bins;
    const float4 *rec;
    const float *background;
    const float *final_Ts;
    const int32_t *final_idx;
    const float *v_img, *v_alpha;
    float *v_colors, *v_opac, *v_xy, *v_xy_abs, *v_conic;
    const uint8_t *blend;  // the forward's blend bytes (16x16 tiles), or null
};

// Global gradient slot of field f (G_R..G_Y) of list entry g whose colour
// gradient goes to Gaussian gc.
__device__ __forceinline__ float *grad_field(const RasterBwdArgs &a, int f, int g, int gc) {
    return f < 3 ? a.v_colors + 3 * (size_t)gc + f
         : f < 6 ? a.v_conic + 3 * (size_t)g + (f - 3)
                 : a.v_xy + 2 * (size_t)g + (f - 6);
}

// kScene: the color and opacity gradients go to the Gaussian whose index the
// record carries in r2.w (batched views of shared scenes) instead of the list
// entry's own index.
template <bool kAbs, bool kScene>
__device__ __forceinline__ void bwd_tile(const RasterBwdArgs &a, const TileCtx &c) {
    __shared__ float4 s_r0[kMaxTile];
    __shared__ float4 s_r1[kMaxTile];
    __shared__ float s_blue[kMaxTile];
    __shared__ unsigned s_mask[kMaxTile];
    __shared__ int s_gid[kMaxTile];
    __shared__ int s_cidx[kScene ? kMaxTile : 1];
    __shared__ int s_wmax[kMaxWarps];
    __shared__ float4 s_rect[kMaxWarps];
    __shared__ uint8_t s_list[kMaxWarps][kMaxTile];

    const int tile = c.tile;
    const int tr = threadIdx.x;
    const int bsize = a.bw * a.bw;
    const int lane = tr & 31, warp = tr >> 5, nwarps = (bsize + 31) >> 5;
    int tx, ty;
    pixel_of(tr, a.bw, tx, ty);
    const unsigned i = c.oy + ty;
    const unsigned j = c.ox + tx;
    const float px = (float)j + 0.5f;
    const float py = (float)i + 0.5f;
    const bool inside = i < c.height && j < c.width;
    // backward.cu:184: out-of-image threads read the last pixel
    const size_t npix = (size_t)c.width * c.height;
    const size_t pix = c.pix_base + min((size_t)i * c.width + j, npix - 1);
    const float3 bg = c.bg;

    if (a.count.get() == 0) return;  // lib/ops.cu:184-186: gradients stay zero
    const float T_final = a.final_Ts[pix];
    float T = T_final;
    const int bin_final = inside ? a.final_idx[pix] : 0;
    const float3 v_out = make_float3(a.v_img[3 * pix], a.v_img[3 * pix + 1], a.v_img[3 * pix + 2]);
    // S . v_out and T_final (v_out_alpha - bg . v_out): see BwdPixel
    float sv = 0.f;
    const float kb = T_final * (a.v_alpha[pix] - (bg.x * v_out.x + bg.y * v_out.y + bg.z * v_out.z));
    const int2 range = a.bins[tile];

    // a partial last warp (bw*bw not a multiple of 32) votes over its lanes only
    const unsigned wmask = (warp == nwarps - 1 && (bsize & 31)) ? ((1u << (bsize & 31)) - 1u)
                                                                : 0xffffffffu;
    const int warp_bin_final = __reduce_max_sync(wmask, bin_final);
    if (lane == 0) s_wmax[warp] = warp_bin_final;
    if (tr < nwarps) s_rect[tr] = warp_rect(tr, a.bw, bsize, (float)c.ox, (float)c.oy);
    __syncthreads();
    int block_max = 0;
    for (int w = 0; w < nwarps; ++w) block_max = max(block_max, s_wmax[w]);
    // no pixel of the tile looks at entries past block_max
    const int top = min(range.y - 1, block_max);

    for (int batch_end = top; batch_end >= range.x; batch_end -= bsize) {
        __syncthreads();  // previous batch fully flushed
        const int idx = batch_end - tr;
        if (idx >= range.x) {
            const int g = a.ids[idx];
            if (g >= 0 && g < a.n) {
                const float4 r0 = a.rec[3 * (size_t)g];
                const float4 r1 = a.rec[3 * (size_t)g + 1];
                const float4 r2 = a.rec[3 * (size_t)g + 2];
                s_gid[tr] = g;
                if (kScene) s_cidx[tr] = __float_as_int(r2.w);
                s_r0[tr] = r0;
                s_r1[tr] = r1;
                s_blue[tr] = r2.x;
                s_mask[tr] = warp_mask(r0, r2, s_rect, nwarps);
            } else {  // corrupt list entry: never contributes, never flushed
                raise_status(a.status, DEV_BAD_ID);
                s_gid[tr] = 0;
                s_mask[tr] = 0u;
            }
        }
        __syncthreads();
        const int n = min(bsize, batch_end + 1 - range.x);
        const int cnt = warp_list(s_mask, max(0, batch_end - warp_bin_final), n, warp, lane, wmask,
                                  s_list[warp]);
        for (int k = 0; k < cnt; ++k) {
            const int t = s_list[warp][k];
            bool valid = inside && (batch_end - t <= bin_final);
            float alpha = 0.f, opac = 0.f, vis = 0.f;
            float2 delta = make_float2(0.f, 0.f);
            float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
            if (valid) {
                r0 = s_r0[t];
                r1 = s_r1[t];
                opac = r1.y;
                delta = make_float2(r0.x - px, r0.y - py);
                const float sigma = falloff(r0.z, r0.w, r1.x, delta.x, delta.y);
                vis = __expf(-sigma);
                alpha = fminf(0.99f, opac * vis);
                if (sigma < 0.f || alpha < 1.f / 255.f) valid = false;
            }
            const unsigned vmask = __ballot_sync(wmask, valid);
            if (!vmask) continue;
            float g8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float g_op = 0.f, g_ax = 0.f, g_ay = 0.f;
            if (valid) {
                const float ra = __fdividef(1.f, 1.f - alpha);  // fast reciprocal, as bwd16_tile
                T *= ra;
                const float fac = alpha * T;
                g8[G_R] = fac * v_out.x;
                g8[G_G] = fac * v_out.y;
                g8[G_B] = fac * v_out.z;
                const float cr = r1.z, cg = r1.w, cb = s_blue[t];
                const float cv = cr * v_out.x + cg * v_out.y + cb * v_out.z;
                const float v_a = T * cv + (kb - sv) * ra;
                sv += fac * cv;
                const float v_sigma = -opac * vis * v_a;
                g8[G_CA] = 0.5f * v_sigma * delta.x * delta.x;
                g8[G_CB] = v_sigma * delta.x * delta.y;
                g8[G_CC] = 0.5f * v_sigma * delta.y * delta.y;
                g8[G_X] = v_sigma * (r0.z * delta.x + r0.w * delta.y);
                g8[G_Y] = v_sigma * (r0.w * delta.x + r1.x * delta.y);
                g_op = vis * v_a;
                if (kAbs) {
                    g_ax = fabsf(g8[G_X]);
                    g_ay = fabsf(g8[G_Y]);
                }
            }
            // warp sums straight to global memory (see raster_bwd16_kernel)
            const int g = s_gid[t];
            const int gc = kScene ? s_cidx[t] : g;
            if (wmask == 0xffffffffu && __popc(vmask) > kFewLanes) {
                float sop;
                const float s8 = warp_sum9_transposed(g8, g_op, lane, &sop);
                if ((lane & 3) == 0) atomicAdd(grad_field(a, lane >> 2, g, gc), s8);
                if (lane == 0) atomicAdd(&a.v_opac[gc], sop);
                if (kAbs) {
                    const float sax = warp_sum(g_ax), say = warp_sum(g_ay);
                    if (lane == 0) {
                        atomicAdd(&a.v_xy_abs[2 * (size_t)g + 0], sax);
                        atomicAdd(&a.v_xy_abs[2 * (size_t)g + 1], say);
                    }
                }
            } else if (valid) {
#pragma unroll
                for (int f = 0; f < 8; ++f) atomicAdd(grad_field(a, f, g, gc), g8[f]);
                atomicAdd(&a.v_opac[gc], g_op);
                if (kAbs) {
                    atomicAdd(&a.v_xy_abs[2 * (size_t)g + 0], g_ax);
                    atomicAdd(&a.v_xy_abs[2 * (size_t)g + 1], g_ay);
                }
            }
        }
    }
}

template <bool kAbs>
__global__ void __launch_bounds__(kMaxTile) raster_bwd_kernel(RasterBwdArgs a) {
    bwd_tile<kAbs, false>(a, grid_tile(a.tiles_x, a.bw, a.width, a.height, a.background));
}

// ---------------------------------------------------------------------------
// Backward for 16x16 tiles: two pixels per thread.  128 threads; warp w owns
// the 8x8 pixel block at ((w & 1) * 8, (w >> 1) * 8), lane l the pixels (x, y)
// and (x, y + 4) with x = l & 7, y = l >> 3 inside it.  Each list entry is
// read from shared memory once per lane and evaluated for both pixels, and one
// warp reduction covers 64 pixels.  Per-pixel arithmetic is unchanged.  (The
// same layout in the forward measured slower than one pixel per thread, which
// is what the forward keeps.)  After the warp reduction the warp's sums go
// straight to global memory, one atomic per field per (warp, Gaussian), as in
// backward.cu:314-340: measured faster here than accumulating per (tile,
// Gaussian) in shared memory and flushing after each batch (the global
// reduction pipe is lightly loaded; the shared accumulators, their zeroing
// and the flush barrier cost more).

constexpr int kT16Threads = 128;
constexpr int kT16Warps = 4;
constexpr int kT16Batch = 256;


// Per-pixel state of the backward pass (backward.cu:181-211), for the two
// pixels of a lane: component x is pixel (x, y), component y pixel (x, y + 4).
// The running color sum S of backward.cu:193 enters the alpha cotangent
// only as S . v_out, and the background and alpha-image terms only as
// T_final (v_out_alpha - bg . v_out); both are carried as scalars:
//   v_alpha = T (c . v_out) + (T_final (v_out_alpha - bg . v_out) - S . v_out) / (1 - alpha)
// which is the reference's expression regrouped.
//
// The two pixels run the same arithmetic, so it is written with Blackwell's
// paired fp32 instructions (FFMA2/FMUL2/FADD2 through __ffma2_rn, __fmul2_rn,
// __fadd2_rn): one instruction issues both pixels' operation, each component
// rounded exactly as the scalar operation would be.  The falloff keeps the
// forward's roundings (falloff() in splat_math.cuh), so both passes make the
// same contribution decisions.
struct BwdPair {
    float2 py;
    bool inside0, inside1;
    int bin0, bin1;
    float2 T, sv, kb;  // transmittance, S . v_out, T_final (v_out_alpha - bg . v_out)
    float2 vx, vy, vz; // v_out
};

template <bool kAbs, bool kScene, bool kBlend = false>
__device__ __forceinline__ void bwd16_tile(const RasterBwdArgs &a, const TileCtx &c) {
    __shared__ float4 s_r0[kT16Batch];
    __shared__ float4 s_r1[kT16Batch];
    __shared__ float s_blue[kT16Batch];
    __shared__ unsigned s_mask[kT16Batch];
    __shared__ int s_gid[kT16Batch];
    __shared__ int s_cidx[kScene ? kT16Batch : 1];
    __shared__ int s_wmax[kT16Warps];
    __shared__ float4 s_rect[kT16Warps];
    __shared__ uint8_t s_list[kT16Warps][kT16Batch];

    const int tile = c.tile;
    const int tr = threadIdx.x, lane = tr & 31, warp = tr >> 5;
    const unsigned j = c.ox + ((warp & 1) << 3) + (lane & 7);
    const unsigned i0 = c.oy + ((warp >> 1) << 3) + (lane >> 3);
    const float px = (float)j + 0.5f;
    if (a.count.get() == 0) return;  // lib/ops.cu:184-186: gradients stay zero
    const size_t npix = (size_t)c.width * c.height;
    const float3 bg = c.bg;
    BwdPair P;
    {
        float Tf[2], kb[2], vx[2], vy[2], vz[2];
        bool in[2];
        int bin[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const unsigned i = i0 + 4 * q;
            in[q] = i < c.height && j < c.width;
            // backward.cu:184: out-of-image threads read the last pixel
            const size_t pix = c.pix_base + min((size_t)i * c.width + j, npix - 1);
            Tf[q] = a.final_Ts[pix];
            bin[q] = in[q] ? a.final_idx[pix] : 0;
            vx[q] = a.v_img[3 * pix];
            vy[q] = a.v_img[3 * pix + 1];
            vz[q] = a.v_img[3 * pix + 2];
            kb[q] = Tf[q] * (a.v_alpha[pix] - (bg.x * vx[q] + bg.y * vy[q] + bg.z * vz[q]));
        }
        P.py = make_float2((float)i0 + 0.5f, (float)(i0 + 4) + 0.5f);
        P.inside0 = in[0];
        P.inside1 = in[1];
        P.bin0 = bin[0];
        P.bin1 = bin[1];
        P.T = make_float2(Tf[0], Tf[1]);
        P.sv = make_float2(0.f, 0.f);
        P.kb = make_float2(kb[0], kb[1]);
        P.vx = make_float2(vx[0], vx[1]);
        P.vy = make_float2(vy[0], vy[1]);
        P.vz = make_float2(vz[0], vz[1]);
    }
    const int2 range = a.bins[tile];
    const int warp_bin_final = __reduce_max_sync(0xffffffffu, max(P.bin0, P.bin1));
    if (lane == 0) s_wmax[warp] = warp_bin_final;
    if (tr < kT16Warps) s_rect[tr] = warp_rect16(tr, (float)c.ox, (float)c.oy);
    __syncthreads();
    int block_max = 0;
#pragma unroll
    for (int w = 0; w < kT16Warps; ++w) block_max = max(block_max, s_wmax[w]);
    const int top = min(range.y - 1, block_max);
    const float2 neg_py = make_float2(-P.py.x, -P.py.y);

    for (int batch_end = top; batch_end >= range.x; batch_end -= kT16Batch) {
        __syncthreads();  // previous batch fully flushed
        for (int e = tr; e < kT16Batch; e += kT16Threads) {
            const int idx = batch_end - e;
            if (idx >= range.x) {
                // with the forward's blend bytes, an entry that no warp
                // passed is never gathered, and the bytes replace the box test
                const unsigned bm = kBlend ? (unsigned)a.blend[idx] : 0u;
                if (kBlend && bm == 0u) {
                    s_mask[e] = 0u;
                    continue;
                }
                const int g = a.ids[idx];
                if (g >= 0 && g < a.n) {
                    const float4 r0 = a.rec[3 * (size_t)g];
                    const float4 r1 = a.rec[3 * (size_t)g + 1];
                    const float4 r2 = a.rec[3 * (size_t)g + 2];
                    s_gid[e] = g;
                    if (kScene) s_cidx[e] = __float_as_int(r2.w);
                    s_r0[e] = r0;
                    s_r1[e] = r1;
                    s_blue[e] = r2.x;
                    s_mask[e] = kBlend ? bm : warp_mask(r0, r2, s_rect, kT16Warps);
                } else {  // corrupt list entry: never contributes, never flushed
                    raise_status(a.status, DEV_BAD_ID);
                    s_gid[e] = 0;
                    s_mask[e] = 0u;
                }
            }
        }
        __syncthreads();
        const int n = min(kT16Batch, batch_end + 1 - range.x);
        const int cnt = warp_list(s_mask, max(0, batch_end - warp_bin_final), n, warp, lane,
                                  0xffffffffu, s_list[warp]);
        for (int k = 0; k < cnt; ++k) {
            const int t = s_list[warp][k];
            const float4 r0 = s_r0[t];
            const float4 r1 = s_r1[t];
            const float opac = r1.y;
            const float dx = r0.x - px;
            const float2 dy = add2(f2(r0.y), neg_py);
            const float2 sigma = falloff2(r0.z, r0.w, r1.x, dx, dy);
            const float vis0 = __expf(-sigma.x), vis1 = __expf(-sigma.y);
            const float2 ov = mul2(f2(opac), make_float2(vis0, vis1));
            const float al0 = fminf(0.99f, ov.x), al1 = fminf(0.99f, ov.y);
            const int back = batch_end - t;
            const bool valid0 = P.inside0 && back <= P.bin0 && !(sigma.x < 0.f || al0 < 1.f / 255.f);
            const bool valid1 = P.inside1 && back <= P.bin1 && !(sigma.y < 0.f || al1 < 1.f / 255.f);
            const unsigned vmask = __ballot_sync(0xffffffffu, valid0 || valid1);
            if (!vmask) continue;
            // a pixel that does not contribute runs with alpha = vis = 0: its
            // T and S stay unchanged (1 / (1 - 0) = 1) and every term it adds
            // is zero
            const float2 al = make_float2(valid0 ? al0 : 0.f, valid1 ? al1 : 0.f);
            const float2 vis = make_float2(valid0 ? vis0 : 0.f, valid1 ? vis1 : 0.f);
            const float2 oma = fma2(al, f2(-1.f), f2(1.f));  // 1 - alpha, one rounding
            // 1 / (1 - alpha) with the fast reciprocal (<= 2 ulp; the
            // reference's IEEE division costs several times as many
            // instructions): the recomputed T and the gradients differ from
            // the reference's by a few ulp, 1 - alpha lies in [0.01, 1)
            const float2 ra = make_float2(__fdividef(1.f, oma.x), __fdividef(1.f, oma.y));
            P.T = mul2(P.T, ra);
            const float2 fac = mul2(al, P.T);
            const float cr = r1.z, cg = r1.w, cb = s_blue[t];
            const float2 cv = fma2(f2(cr), P.vx, fma2(f2(cg), P.vy, mul2(f2(cb), P.vz)));
            const float2 v_a = fma2(P.T, cv, mul2(fma2(P.sv, f2(-1.f), P.kb), ra));
            P.sv = fma2(fac, cv, P.sv);
            const float2 u = mul2(vis, v_a);            // opacity cotangent, per pixel
            const float2 v_sigma = mul2(f2(-opac), u);  // -opac vis v_alpha
            const float2 w = mul2(v_sigma, f2(dx));     // v_sigma dx
            const float2 z = mul2(v_sigma, dy);         // v_sigma dy
            const float2 gx = fma2(f2(r0.z), w, mul2(f2(r0.w), z));
            const float2 gy = fma2(f2(r0.w), w, mul2(f2(r1.x), z));
            float g8[8];
            g8[G_R] = hsum(mul2(fac, P.vx));
            g8[G_G] = hsum(mul2(fac, P.vy));
            g8[G_B] = hsum(mul2(fac, P.vz));
            g8[G_CA] = hsum(mul2(w, f2(0.5f * dx)));
            g8[G_CB] = hsum(mul2(w, dy));
            g8[G_CC] = hsum(mul2(z, mul2(f2(0.5f), dy)));
            g8[G_X] = hsum(gx);
            g8[G_Y] = hsum(gy);
            const float g_op = hsum(u);
            float g_ax = 0.f, g_ay = 0.f;
            if (kAbs) {
                g_ax = fabsf(gx.x) + fabsf(gx.y);
                g_ay = fabsf(gy.x) + fabsf(gy.y);
            }
            const int g = s_gid[t];
            const int gc = kScene ? s_cidx[t] : g;
            if (__popc(vmask) > kFewLanes) {
                float sop;
                const float s8 = warp_sum9_transposed(g8, g_op, lane, &sop);
                if ((lane & 3) == 0) atomicAdd(grad_field(a, lane >> 2, g, gc), s8);
                if (lane == 0) atomicAdd(&a.v_opac[gc], sop);
                if (kAbs) {
                    const float sax = warp_sum(g_ax), say = warp_sum(g_ay);
                    if (lane == 0) {
                        atomicAdd(&a.v_xy_abs[2 * (size_t)g + 0], sax);
                        atomicAdd(&a.v_xy_abs[2 * (size_t)g + 1], say);
                    }
                }
            } else if (valid0 || valid1) {
#pragma unroll
                for (int f = 0; f < 8; ++f) atomicAdd(grad_field(a, f, g, gc), g8[f]);
                atomicAdd(&a.v_opac[gc], g_op);
                if (kAbs) {
                    atomicAdd(&a.v_xy_abs[2 * (size_t)g + 0], g_ax);
                    atomicAdd(&a.v_xy_abs[2 * (size_t)g + 1], g_ay);
                }
            }
        }
    }
}

template <bool kAbs, bool kBlend>
__global__ void __launch_bounds__(kT16Threads) raster_bwd16_kernel(RasterBwdArgs a) {
    bwd16_tile<kAbs, false, kBlend>(a, grid_tile(a.tiles_x, 16, a.width, a.height,
                                                 a.background));
}

// ---------------------------------------------------------------------------
// Batched views: persistent blocks take `chunk` tiles at a time from a work
// list (longest tile list first) through an atomic counter; each tile's view
// comes from the view table.

struct BatchTiles {
    const int32_t *order;
    int ntiles;
    int chunk;
    int *next;  // work counter, zero at launch
    const splat_view *views;
    int nviews;
};

__device__ __forceinline__ TileCtx view_tile(const BatchTiles &b, int tile, unsigned bw) {
    const splat_view &v = b.views[view_by_tile(b.views, b.nviews, (uint32_t)tile)];
    const unsigned local = (unsigned)tile - v.tile_base;
    TileCtx c;
    c.tile = tile;
    c.ox = (local % v.tiles_x) * bw;
    c.oy = (local / v.tiles_x) * bw;
    c.width = v.img_width;
    c.height = v.img_height;
    c.pix_base = (size_t)v.pixel_base;
    c.bg = make_float3(v.background[0], v.background[1], v.background[2]);
    return c;
}

// Calls body(tile context) for every tile of the work list, with the block
// synchronised between tiles.
template <class Body>
__device__ __forceinline__ void for_each_work_tile(const BatchTiles &b, unsigned bw, Body body) {
    __shared__ int s_first;
    for (;;) {
        __syncthreads();  // the previous tile is done with shared memory
        if (threadIdx.x == 0) s_first = atomicAdd(b.next, b.chunk);
        __syncthreads();
        const int first = s_first;
        if (first >= b.ntiles) return;
        const int last = min(first + b.chunk, b.ntiles);
        for (int it = first; it < last; ++it) {
            if (it > first) __syncthreads();
            const int tile = b.order[it];
            if (tile >= 0 && tile < b.ntiles) body(view_tile(b, tile, bw));
        }
    }
}

template <bool kLoss>
__global__ void __launch_bounds__(kMaxTile, 5) raster_fwd_batch_kernel(RasterFwdArgs a, BatchTiles b) {
    for_each_work_tile(b, a.bw, [&](const TileCtx &c) { fwd_tile<kLoss, kLoss>(a, c); });
}

template <bool kLoss>
__global__ void __launch_bounds__(kF16Threads) raster_fwd16_batch_kernel(RasterFwdArgs a,
                                                                          BatchTiles b) {
    for_each_work_tile(b, 16, [&](const TileCtx &c) { fwd16_tile<kLoss, kLoss>(a, c); });
}

__global__ void __launch_bounds__(kMaxTile) raster_bwd_batch_kernel(RasterBwdArgs a, BatchTiles b) {
    for_each_work_tile(b, a.bw, [&](const TileCtx &c) { bwd_tile<false, true>(a, c); });
}

__global__ void __launch_bounds__(kT16Threads) raster_bwd16_batch_kernel(RasterBwdArgs a,
                                                                          BatchTiles b) {
    for_each_work_tile(b, 16, [&](const TileCtx &c) { bwd16_tile<false, true>(a, c); });
}

// ---------------------------------------------------------------------------
// Host launchers.

int launch_pack(const splat_params &p, const float *xys, const float *conics,
                const float *colors, const float *opac, float *rec, cudaStream_t s) {
    PackArgs a;
    a.n = (int)p.num_points;
    a.xys = xys; a.conics = conics; a.colors = colors; a.opac = opac;
    a.rec = reinterpret_cast<float4 *>(rec);
    if (a.n == 0) return SPLAT_OK;
    pack_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a);
    return check_launch("pack_kernel");
}

int launch_batch_pack(const splat_batch &b, const float *xys, const float *conics,
                      const float *colors, const float *opac, float *rec, cudaStream_t s) {
    PackArgs a;
    a.n = (int)b.num_entries;
    a.xys = xys; a.conics = conics; a.colors = colors; a.opac = opac;
    a.rec = reinterpret_cast<float4 *>(rec);
    if (a.n == 0) return SPLAT_OK;
    pack_batch_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a, b.views, (int)b.num_views);
    return check_launch("pack_batch_kernel");
}

// Resident blocks per SM times the SM count: the persistent grid.
template <class K>
static int persistent_grid(K kernel, int threads, int *grid) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess)
        return check_launch("persistent grid query");
    *grid = std::max(1, sms * std::max(1, per_sm));
    return SPLAT_OK;
}

static BatchTiles batch_tiles(const splat_batch &b, const int32_t *order, int chunk, int *next) {
    BatchTiles t;
    t.order = order;
    t.ntiles = (int)b.num_tiles;
    t.chunk = chunk;
    t.next = next;
    t.views = b.views;
    t.nviews = (int)b.num_views;
    return t;
}

// target / v_img / loss non-null: the per-view L2 loss is fused in.
int launch_batch_raster_fwd(const splat_batch &b, Count count, const int32_t *ids,
                            const int2 *bins, const int32_t *order, const float *rec,
                            float *final_Ts, int32_t *final_idx, float *img, const float *target,
                            float *v_img, float *loss, int chunk, int *next, cudaStream_t s) {
    const bool fused = target != nullptr;
    if (fused && cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess)
        return check_launch("loss memset");
    if (b.num_tiles == 0) return SPLAT_OK;
    if (cudaMemsetAsync(next, 0, sizeof(int), s) != cudaSuccess)
        return check_launch("work counter memset");
    RasterFwdArgs a;
    a.tiles_x = 0; a.width = 0; a.height = 0; a.bw = b.block_width;
    a.n = (int)b.num_entries; a.status = b.device_status;
    a.count = count; a.ids = ids; a.bins = bins;
    a.rec = reinterpret_cast<const float4 *>(rec); a.background = nullptr;
    a.final_Ts = final_Ts; a.final_idx = final_idx; a.img = img;
    a.target = target; a.v_img = v_img; a.loss = loss; a.inv_count = 0.f; a.blend = nullptr;
    const BatchTiles t = batch_tiles(b, order, chunk, next);
    int threads = (int)(b.block_width * b.block_width);
    int grid = 0;
    auto run = [&](auto kernel) -> int {
        if (int rc = persistent_grid(kernel, threads, &grid)) return rc;
        kernel<<<grid, threads, 0, s>>>(a, t);
        return check_launch("raster_fwd_batch_kernel");
    };
    if (b.block_width == 16) {
        threads = kF16Threads;
        return fused ? run(raster_fwd16_batch_kernel<true>) : run(raster_fwd16_batch_kernel<false>);
    }
    return fused ? run(raster_fwd_batch_kernel<true>) : run(raster_fwd_batch_kernel<false>);
}

int launch_batch_raster_bwd(const splat_batch &b, Count count, const int32_t *ids,
                            const int2 *bins, const int32_t *order, const float *rec,
                            const float *final_Ts, const int32_t *final_idx, const float *v_img,
                            const float *v_alpha, float *v_colors, float *v_opac, float *v_xy,
                            float *v_conic, int chunk, int *next, cudaStream_t s) {
    const size_t g = b.num_points, e = b.num_entries;
    if (cudaMemsetAsync(v_colors, 0, g * 3 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_opac, 0, g * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_xy, 0, e * 2 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_conic, 0, e * 3 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(next, 0, sizeof(int), s) != cudaSuccess)
        return check_launch("batch raster_bwd output memset");
    if (count.cap == 0 || b.num_tiles == 0) return SPLAT_OK;
    RasterBwdArgs a;
    a.tiles_x = 0; a.width = 0; a.height = 0; a.bw = b.block_width;
    a.n = (int)b.num_entries; a.status = b.device_status;
    a.count = count; a.ids = ids; a.bins = bins;
    a.rec = reinterpret_cast<const float4 *>(rec); a.background = nullptr;
    a.final_Ts = final_Ts; a.final_idx = final_idx; a.v_img = v_img; a.v_alpha = v_alpha;
    a.v_colors = v_colors; a.v_opac = v_opac; a.v_xy = v_xy; a.v_xy_abs = nullptr;
    a.v_conic = v_conic; a.blend = nullptr;
    const BatchTiles t = batch_tiles(b, order, chunk, next);
    int grid = 0;
    if (b.block_width == 16) {
        if (int rc = persistent_grid(raster_bwd16_batch_kernel, kT16Threads, &grid)) return rc;
        raster_bwd16_batch_kernel<<<grid, kT16Threads, 0, s>>>(a, t);
        return check_launch("raster_bwd16_batch_kernel");
    }
    const int threads = (int)(b.block_width * b.block_width);
    if (int rc = persistent_grid(raster_bwd_batch_kernel, threads, &grid)) return rc;
    raster_bwd_batch_kernel<<<grid, threads, 0, s>>>(a, t);
    return check_launch("raster_bwd_batch_kernel");
}

// ---------------------------------------------------------------------------
// Work counts for the compute roofline (diagnostic; not on the step path).
// One block per tile, one thread per pixel (row-major), every list entry in
// order, with the reference's per-pixel semantics and no culling:
//   [0] pairs the forward evaluates: per pixel, entries up to and including
//       the one that saturates it (forward.cu:380-455);
//   [1] pairs the backward evaluates: entries up to the pixel's final_idx
//       (backward.cu:240-262);
//   [2] of those, the contributing ones (sigma >= 0 and alpha >= 1/255);
//   [3] (tile, Gaussian) pairs with at least one contributing pixel (the
//       granularity of the reference's gradient atomics, backward.cu:314-340).

struct CountArgs {
    unsigned tiles_x, width, height, bw;
    int n;
    Count count;
    const int32_t *ids;
    const int2 *bins;
    const float4 *rec;
    const int32_t *final_idx;
    unsigned long long *counts;
};

__global__ void __launch_bounds__(kMaxTile) count_pairs_kernel(CountArgs a) {
    __shared__ unsigned s_sum[3][kMaxWarps];
    const int tile = (int)(blockIdx.y * a.tiles_x + blockIdx.x);
    const int tr = threadIdx.x, lane = tr & 31, warp = tr >> 5;
    const int bsize = (int)(a.bw * a.bw), nwarps = (bsize + 31) >> 5;
    const unsigned i = blockIdx.y * a.bw + tr / a.bw, j = blockIdx.x * a.bw + tr % a.bw;
    const bool inside = i < a.height && j < a.width;
    const float px = (float)j + 0.5f, py = (float)i + 0.5f;
    if (a.count.get() == 0) return;
    const int2 range = a.bins[tile];
    const int fidx = inside ? a.final_idx[(size_t)i * a.width + j] : -1;
    bool done = !inside;
    float T = 1.f;
    unsigned e_fwd = 0, e_bwd = 0, e_valid = 0, e_tile = 0;
    for (int e = range.x; e < range.y; ++e) {
        const int g = a.ids[e];
        bool valid = false;
        if (g >= 0 && g < a.n && inside && (!done || e <= fidx)) {
            const float4 r0 = a.rec[3 * (size_t)g], r1 = a.rec[3 * (size_t)g + 1];
            const float sigma = falloff(r0.z, r0.w, r1.x, r0.x - px, r0.y - py);
            const float vis = __expf(-sigma);
            if (!done) {
                ++e_fwd;
                const float alpha = fminf(0.999f, r1.y * vis);
                if (sigma >= 0.f && alpha >= 1.f / 255.f) {
                    const float next_T = T * (1.f - alpha);
                    if (next_T <= 1e-4f) done = true;
                    else T = next_T;
                }
            }
            if (e <= fidx) {
                ++e_bwd;
                const float alpha = fminf(0.99f, r1.y * vis);
                valid = sigma >= 0.f && alpha >= 1.f / 255.f;
                e_valid += valid;
            }
        }
        if (__syncthreads_or(valid) && tr == 0) ++e_tile;
    }
    unsigned v[3] = {e_fwd, e_bwd, e_valid};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        unsigned x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) s_sum[q][warp] = x;
    }
    __syncthreads();
    if (tr < 3) {
        unsigned long long t = 0;
        for (int w = 0; w < nwarps; ++w) t += s_sum[tr][w];
        atomicAdd(&a.counts[tr], t);
    }
    if (tr == 0) atomicAdd(&a.counts[3], (unsigned long long)e_tile);
}

int launch_count_pairs(const splat_params &p, Count count, const int32_t *ids, const int2 *bins,
                       const float *rec, const int32_t *final_idx, unsigned long long *counts,
                       cudaStream_t s) {
    if (cudaMemsetAsync(counts, 0, 4 * sizeof(unsigned long long), s) != cudaSuccess)
        return check_launch("count_pairs memset");
    if (count.cap == 0) return SPLAT_OK;
    CountArgs a;
    a.tiles_x = tiles_x(p); a.width = p.img_width; a.height = p.img_height; a.bw = p.block_width;
    a.n = (int)p.num_points; a.count = count; a.ids = ids; a.bins = bins;
    a.rec = reinterpret_cast<const float4 *>(rec); a.final_idx = final_idx; a.counts = counts;
    dim3 grid(tiles_x(p), tiles_y(p));
    count_pairs_kernel<<<grid, p.block_width * p.block_width, 0, s>>>(a);
    return check_launch("count_pairs_kernel");
}

// target / v_img / loss non-null: the L2 loss is fused into the epilogue.
int launch_raster_fwd(const splat_params &p, Count count, const int32_t *ids,
                      const int2 *bins, const float *rec, const float *background,
                      float *final_Ts, int32_t *final_idx, float *img, const float *target,
                      float *v_img, float *loss, uint8_t *blend, cudaStream_t s) {
    RasterFwdArgs a;
    a.tiles_x = tiles_x(p); a.width = p.img_width; a.height = p.img_height; a.bw = p.block_width;
    a.n = (int)p.num_points; a.status = p.device_status;
    a.count = count; a.ids = ids; a.bins = bins;
    a.rec = reinterpret_cast<const float4 *>(rec); a.background = background;
    a.final_Ts = final_Ts; a.final_idx = final_idx; a.img = img;
    a.target = target; a.v_img = v_img; a.loss = loss; a.blend = blend;
    const long long npix3 = 3ll * p.img_width * p.img_height;
    a.inv_count = npix3 > 0 ? 1.f / (float)npix3 : 0.f;
    const bool fused = target != nullptr;
    if (fused && cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess)
        return check_launch("loss memset");
    dim3 grid(tiles_x(p), tiles_y(p));
    const unsigned threads = p.block_width * p.block_width;
    if (p.block_width == 16) {
        if (blend) {
            if (fused) raster_fwd16_kernel<true, true><<<grid, kF16Threads, 0, s>>>(a);
            else raster_fwd16_kernel<false, true><<<grid, kF16Threads, 0, s>>>(a);
        } else {
            if (fused) raster_fwd16_kernel<true, false><<<grid, kF16Threads, 0, s>>>(a);
            else raster_fwd16_kernel<false, false><<<grid, kF16Threads, 0, s>>>(a);
        }
    } else {
        if (fused) raster_fwd_kernel<true><<<grid, threads, 0, s>>>(a);
        else raster_fwd_kernel<false><<<grid, threads, 0, s>>>(a);
    }
    return check_launch("raster_fwd_kernel");
}

int launch_raster_bwd(const splat_params &p, Count count, const int32_t *ids,
                      const int2 *bins, const float *rec, const float *background,
                      const float *final_Ts, const int32_t *final_idx, const float *v_img,
                      const float *v_alpha, float *v_colors, float *v_opac, float *v_xy,
                      float *v_xy_abs, float *v_conic, const uint8_t *blend, cudaStream_t s) {
    const size_t n = p.num_points;
    // outputs are sums: start from zero (lib/ops.cu:534-572); with no
    // Gaussians there is nothing to clear and nothing to rasterize
    if (n == 0) return SPLAT_OK;
    if (cudaMemsetAsync(v_colors, 0, n * 3 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_opac, 0, n * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_xy, 0, n * 2 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_conic, 0, n * 3 * sizeof(float), s) != cudaSuccess ||
        (v_xy_abs && cudaMemsetAsync(v_xy_abs, 0, n * 2 * sizeof(float), s) != cudaSuccess))
        return check_launch("raster_bwd output memset");
    if (count.cap == 0) return SPLAT_OK;  // lib/ops.cu:184-186
    RasterBwdArgs a;
    a.tiles_x = tiles_x(p); a.width = p.img_width; a.height = p.img_height; a.bw = p.block_width;
    a.n = (int)p.num_points; a.status = p.device_status;
    a.count = count; a.ids = ids; a.bins = bins;
    a.rec = reinterpret_cast<const float4 *>(rec); a.background = background;
    a.final_Ts = final_Ts; a.final_idx = final_idx; a.v_img = v_img; a.v_alpha = v_alpha;
    a.v_colors = v_colors; a.v_opac = v_opac; a.v_xy = v_xy; a.v_xy_abs = v_xy_abs;
    a.v_conic = v_conic; a.blend = blend;
    dim3 grid(tiles_x(p), tiles_y(p));
    const unsigned threads = p.block_width * p.block_width;
    const bool wide = p.block_width == 16;
    if (wide) {
        if (blend) {
            if (v_xy_abs) raster_bwd16_kernel<true, true><<<grid, kT16Threads, 0, s>>>(a);
            else raster_bwd16_kernel<false, true><<<grid, kT16Threads, 0, s>>>(a);
        } else {
            if (v_xy_abs) raster_bwd16_kernel<true, false><<<grid, kT16Threads, 0, s>>>(a);
            else raster_bwd16_kernel<false, false><<<grid, kT16Threads, 0, s>>>(a);
        }
        return check_launch("raster_bwd16_kernel");
    }
    if (v_xy_abs)
        raster_bwd_kernel<true><<<grid, threads, 0, s>>>(a);
    else
        raster_bwd_kernel<false><<<grid, threads, 0, s>>>(a);
    return check_launch("raster_bwd_kernel");
}

}  // namespace splat
