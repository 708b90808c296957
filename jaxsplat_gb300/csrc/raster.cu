// raster.cu -- tile rasterizer, forward and backward.
//
// One block per tile, one thread per pixel (block = bw x bw, bw <= 16).
// Per-pixel arithmetic is the reference's (forward.cu:339-462,
// backward.cu:153-343), evaluated in the same order so that final_idx and the
// image are bit-identical; what differs is how the work is organised:
//   forward  - batches are staged as packed float4 records (x, y, opacity,
//              color.r) and (conic a, b, c, id) so that a batch entry is two
//              shared-memory vector loads; colors are staged too.
//   backward - the block starts at the largest final_idx of its pixels
//              instead of the end of the tile list; per-Gaussian partial sums
//              are reduced across the warp with a transposed butterfly (9
//              shuffles for 8 values instead of 40), accumulated across the
//              block's warps in shared memory and flushed with one global
//              atomic per (tile, Gaussian, field) instead of one per warp.
#include "splat_internal.cuh"
#include "splat_math.cuh"

namespace splat {

constexpr int kMaxTile = 256;  // bw * bw <= 256

struct RasterFwdArgs {
    unsigned tiles_x, width, height, bw;
    int n;
    uint32_t *status;
    long long count;
    const int32_t *ids;
    const int2 *bins;
    const float *xys, *conics, *colors, *opac, *background;
    float *final_Ts;
    int32_t *final_idx;
    float *img;
};

__global__ void __launch_bounds__(kMaxTile) raster_fwd_kernel(RasterFwdArgs a) {
    __shared__ float4 s_xyoc[kMaxTile];  // x, y, opacity, red
    __shared__ float4 s_con[kMaxTile];   // conic a, b, c, green
    __shared__ float s_blue[kMaxTile];
    const int tile = blockIdx.y * a.tiles_x + blockIdx.x;
    const unsigned i = blockIdx.y * a.bw + threadIdx.y;
    const unsigned j = blockIdx.x * a.bw + threadIdx.x;
    const int tr = threadIdx.y * a.bw + threadIdx.x;
    const int bsize = a.bw * a.bw;
    const float px = (float)j + 0.5f;
    const float py = (float)i + 0.5f;
    const bool inside = i < a.height && j < a.width;
    const size_t pix = (size_t)i * a.width + j;
    const float3 bg = make_float3(a.background[0], a.background[1], a.background[2]);

    if (a.count == 0) {  // lib/ops.cu:119-127: background image, zero T and index
        if (inside) {
            a.final_Ts[pix] = 0.f;
            a.final_idx[pix] = 0;
            a.img[3 * pix] = bg.x;
            a.img[3 * pix + 1] = bg.y;
            a.img[3 * pix + 2] = bg.z;
        }
        return;
    }
    const int2 range = a.bins[tile];
    bool done = !inside;
    float T = 1.f;
    int cur_idx = 0;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    for (int start = range.x; start < range.y; start += bsize) {
        if (__syncthreads_count(done) >= bsize) break;
        const int idx = start + tr;
        if (idx < range.y) {
            const int g = a.ids[idx];
            if (g >= 0 && g < a.n) {
                const float2 xy = *reinterpret_cast<const float2 *>(a.xys + 2 * (size_t)g);
                const float o = a.opac[g];
                const float *c = a.colors + 3 * (size_t)g;
                const float *k = a.conics + 3 * (size_t)g;
                s_xyoc[tr] = make_float4(xy.x, xy.y, o, c[0]);
                s_con[tr] = make_float4(k[0], k[1], k[2], c[1]);
                s_blue[tr] = c[2];
            } else {  // corrupt list entry: a zero-opacity record never contributes
                raise_status(a.status, DEV_BAD_ID);
                s_xyoc[tr] = make_float4(0.f, 0.f, 0.f, 0.f);
                s_con[tr] = make_float4(0.f, 0.f, 0.f, 0.f);
                s_blue[tr] = 0.f;
            }
        }
        __syncthreads();
        const int n = min(bsize, range.y - start);
        for (int t = 0; t < n && !done; ++t) {
            const float4 xo = s_xyoc[t];
            const float4 cc = s_con[t];
            const float dx = xo.x - px, dy = xo.y - py;
            const float sigma = falloff(cc.x, cc.y, cc.z, dx, dy);
            const float alpha = fminf(0.999f, xo.z * __expf(-sigma));
            if (sigma < 0.f || alpha < 1.f / 255.f) continue;
            const float next_T = T * (1.f - alpha);
            if (next_T <= 1e-4f) {
                done = true;
                break;
            }
            const float vis = alpha * T;
            acc.x = acc.x + xo.w * vis;
            acc.y = acc.y + cc.w * vis;
            acc.z = acc.z + s_blue[t] * vis;
            T = next_T;
            cur_idx = start + t;
        }
    }
    if (inside) {
        a.final_Ts[pix] = T;
        a.final_idx[pix] = cur_idx;
        a.img[3 * pix] = acc.x + T * bg.x;
        a.img[3 * pix + 1] = acc.y + T * bg.y;
        a.img[3 * pix + 2] = acc.z + T * bg.z;
    }
}

// ---------------------------------------------------------------------------
// Backward.

// Sum of 8 values over the warp, transposed: on return lane L holds the
// warp total of value (L >> 2) & 7.  `lane` is the caller's lane index (the
// blocks here are two-dimensional, so threadIdx.x is not the lane).
__device__ __forceinline__ float warp_sum8_transposed(const float v[8], int lane) {
    float b[4], c[2];
    const bool u16 = lane & 16, u8 = lane & 8, u4 = lane & 4;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float send = u16 ? v[k] : v[k + 4];
        const float keep = u16 ? v[k + 4] : v[k];
        b[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float send = u8 ? b[k] : b[k + 2];
        const float keep = u8 ? b[k + 2] : b[k];
        c[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const float send = u4 ? c[0] : c[1];
    const float keep = u4 ? c[1] : c[0];
    float d = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    d += __shfl_xor_sync(0xffffffffu, d, 2);
    d += __shfl_xor_sync(0xffffffffu, d, 1);
    return d;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Gradient fields accumulated per staged Gaussian.
enum { G_R, G_G, G_B, G_CA, G_CB, G_CC, G_X, G_Y, G_OP, G_AX, G_AY, G_FIELDS };

struct RasterBwdArgs {
    unsigned tiles_x, width, height, bw;
    int n;
    uint32_t *status;
    long long count;
    const int32_t *ids;
    const int2 *bins;
    const float *xys, *conics, *colors, *opac, *background;
    const float *final_Ts;
    const int32_t *final_idx;
    const float *v_img, *v_alpha;
    float *v_colors, *v_opac, *v_xy, *v_xy_abs, *v_conic;
};

template <bool kAbs>
__global__ void __launch_bounds__(kMaxTile) raster_bwd_kernel(RasterBwdArgs a) {
    __shared__ float4 s_xyo[kMaxTile];  // x, y, opacity, -
    __shared__ float4 s_con[kMaxTile];  // conic a, b, c, -
    __shared__ float4 s_rgb[kMaxTile];  // r, g, b, -
    __shared__ int s_gid[kMaxTile];
    __shared__ float s_acc[kMaxTile][G_FIELDS];
    __shared__ int s_touched[kMaxTile];
    __shared__ int s_wmax[kMaxTile / 32];

    const int tile = blockIdx.y * a.tiles_x + blockIdx.x;
    const unsigned i = blockIdx.y * a.bw + threadIdx.y;
    const unsigned j = blockIdx.x * a.bw + threadIdx.x;
    const int tr = threadIdx.y * a.bw + threadIdx.x;
    const int bsize = a.bw * a.bw;
    const int lane = tr & 31, warp = tr >> 5, nwarps = (bsize + 31) >> 5;
    const float px = (float)j + 0.5f;
    const float py = (float)i + 0.5f;
    const bool inside = i < a.height && j < a.width;
    // backward.cu:184: out-of-image threads read the last pixel
    const size_t npix = (size_t)a.width * a.height;
    const size_t pix = min((size_t)i * a.width + j, npix - 1);
    const float3 bg = make_float3(a.background[0], a.background[1], a.background[2]);

    const float T_final = a.final_Ts[pix];
    float T = T_final;
    float3 buf = make_float3(0.f, 0.f, 0.f);
    const int bin_final = inside ? a.final_idx[pix] : 0;
    const float3 v_out = make_float3(a.v_img[3 * pix], a.v_img[3 * pix + 1], a.v_img[3 * pix + 2]);
    const float v_out_alpha = a.v_alpha[pix];
    const int2 range = a.bins[tile];

    // partial warps (bw not a multiple of the warp size) vote with a full mask
    // over the lanes that exist
    const unsigned wmask = (warp == nwarps - 1 && (bsize & 31)) ? ((1u << (bsize & 31)) - 1u)
                                                                : 0xffffffffu;
    const int warp_bin_final = __reduce_max_sync(wmask, bin_final);
    if (lane == 0) s_wmax[warp] = warp_bin_final;
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
                s_gid[tr] = g;
                const float2 xy = *reinterpret_cast<const float2 *>(a.xys + 2 * (size_t)g);
                s_xyo[tr] = make_float4(xy.x, xy.y, a.opac[g], 0.f);
                const float *k = a.conics + 3 * (size_t)g;
                s_con[tr] = make_float4(k[0], k[1], k[2], 0.f);
                const float *c = a.colors + 3 * (size_t)g;
                s_rgb[tr] = make_float4(c[0], c[1], c[2], 0.f);
            } else {  // corrupt list entry: zero opacity, never valid, never flushed
                raise_status(a.status, DEV_BAD_ID);
                s_gid[tr] = 0;
                s_xyo[tr] = make_float4(0.f, 0.f, 0.f, 0.f);
                s_con[tr] = make_float4(0.f, 0.f, 0.f, 0.f);
                s_rgb[tr] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int f = 0; f < G_FIELDS; ++f) s_acc[tr][f] = 0.f;
        s_touched[tr] = 0;
        __syncthreads();
        const int n = min(bsize, batch_end + 1 - range.x);
        for (int t = max(0, batch_end - warp_bin_final); t < n; ++t) {
            bool valid = inside && (batch_end - t <= bin_final);
            float alpha = 0.f, opac = 0.f, vis = 0.f;
            float2 delta = make_float2(0.f, 0.f);
            float4 con = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                con = s_con[t];
                const float4 xo = s_xyo[t];
                opac = xo.z;
                delta = make_float2(xo.x - px, xo.y - py);
                const float sigma = falloff(con.x, con.y, con.z, delta.x, delta.y);
                vis = __expf(-sigma);
                alpha = fminf(0.99f, opac * vis);
                if (sigma < 0.f || alpha < 1.f / 255.f) valid = false;
            }
            if (!__any_sync(wmask, valid)) continue;
            float g8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float g_op = 0.f, g_ax = 0.f, g_ay = 0.f;
            if (valid) {
                const float ra = 1.f / (1.f - alpha);
                T *= ra;
                const float fac = alpha * T;
                float v_a = 0.f;
                g8[G_R] = fac * v_out.x;
                g8[G_G] = fac * v_out.y;
                g8[G_B] = fac * v_out.z;
                const float4 rgb = s_rgb[t];
                v_a += (rgb.x * T - buf.x * ra) * v_out.x;
                v_a += (rgb.y * T - buf.y * ra) * v_out.y;
                v_a += (rgb.z * T - buf.z * ra) * v_out.z;
                v_a += T_final * ra * v_out_alpha;
                v_a += -T_final * ra * bg.x * v_out.x;
                v_a += -T_final * ra * bg.y * v_out.y;
                v_a += -T_final * ra * bg.z * v_out.z;
                buf.x += rgb.x * fac;
                buf.y += rgb.y * fac;
                buf.z += rgb.z * fac;
                const float v_sigma = -opac * vis * v_a;
                g8[G_CA] = 0.5f * v_sigma * delta.x * delta.x;
                g8[G_CB] = v_sigma * delta.x * delta.y;
                g8[G_CC] = 0.5f * v_sigma * delta.y * delta.y;
                g8[G_X] = v_sigma * (con.x * delta.x + con.y * delta.y);
                g8[G_Y] = v_sigma * (con.y * delta.x + con.z * delta.y);
                g_op = vis * v_a;
                if (kAbs) {
                    g_ax = fabsf(g8[G_X]);
                    g_ay = fabsf(g8[G_Y]);
                }
            }
            if (wmask == 0xffffffffu) {
                const float s8 = warp_sum8_transposed(g8, lane);
                const float sop = warp_sum(g_op);
                if ((lane & 3) == 0) atomicAdd(&s_acc[t][lane >> 2], s8);
                if (lane == 0) {
                    atomicAdd(&s_acc[t][G_OP], sop);
                    s_touched[t] = 1;
                }
                if (kAbs) {
                    const float sax = warp_sum(g_ax), say = warp_sum(g_ay);
                    if (lane == 0) {
                        atomicAdd(&s_acc[t][G_AX], sax);
                        atomicAdd(&s_acc[t][G_AY], say);
                    }
                }
            } else if (valid) {
                // partial warp: plain shared atomics per lane
#pragma unroll
                for (int f = 0; f < 8; ++f) atomicAdd(&s_acc[t][f], g8[f]);
                atomicAdd(&s_acc[t][G_OP], g_op);
                if (kAbs) {
                    atomicAdd(&s_acc[t][G_AX], g_ax);
                    atomicAdd(&s_acc[t][G_AY], g_ay);
                }
                s_touched[t] = 1;
            }
        }
        __syncthreads();
        if (idx >= range.x && s_touched[tr]) {
            const int g = s_gid[tr];
            const float *acc = s_acc[tr];
            atomicAdd(&a.v_colors[3 * (size_t)g + 0], acc[G_R]);
            atomicAdd(&a.v_colors[3 * (size_t)g + 1], acc[G_G]);
            atomicAdd(&a.v_colors[3 * (size_t)g + 2], acc[G_B]);
            atomicAdd(&a.v_conic[3 * (size_t)g + 0], acc[G_CA]);
            atomicAdd(&a.v_conic[3 * (size_t)g + 1], acc[G_CB]);
            atomicAdd(&a.v_conic[3 * (size_t)g + 2], acc[G_CC]);
            atomicAdd(&a.v_xy[2 * (size_t)g + 0], acc[G_X]);
            atomicAdd(&a.v_xy[2 * (size_t)g + 1], acc[G_Y]);
            atomicAdd(&a.v_opac[g], acc[G_OP]);
            if (kAbs) {
                atomicAdd(&a.v_xy_abs[2 * (size_t)g + 0], acc[G_AX]);
                atomicAdd(&a.v_xy_abs[2 * (size_t)g + 1], acc[G_AY]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host launchers.

int launch_raster_fwd(const splat_params &p, long long count, const int32_t *ids,
                      const int2 *bins, const float *xys, const float *conics,
                      const float *colors, const float *opac, const float *background,
                      float *final_Ts, int32_t *final_idx, float *img, cudaStream_t s) {
    RasterFwdArgs a;
    a.tiles_x = tiles_x(p); a.width = p.img_width; a.height = p.img_height; a.bw = p.block_width;
    a.n = (int)p.num_points; a.status = p.device_status;
    a.count = count; a.ids = ids; a.bins = bins;
    a.xys = xys; a.conics = conics; a.colors = colors; a.opac = opac; a.background = background;
    a.final_Ts = final_Ts; a.final_idx = final_idx; a.img = img;
    dim3 grid(tiles_x(p), tiles_y(p)), block(p.block_width, p.block_width);
    raster_fwd_kernel<<<grid, block, 0, s>>>(a);
    return check_launch("raster_fwd_kernel");
}

int launch_raster_bwd(const splat_params &p, long long count, const int32_t *ids,
                      const int2 *bins, const float *xys, const float *conics,
                      const float *colors, const float *opac, const float *background,
                      const float *final_Ts, const int32_t *final_idx, const float *v_img,
                      const float *v_alpha, float *v_colors, float *v_opac, float *v_xy,
                      float *v_xy_abs, float *v_conic, cudaStream_t s) {
    const size_t n = p.num_points;
    // outputs are sums: start from zero (lib/ops.cu:534-572)
    if (cudaMemsetAsync(v_colors, 0, n * 3 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_opac, 0, n * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_xy, 0, n * 2 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(v_conic, 0, n * 3 * sizeof(float), s) != cudaSuccess ||
        (v_xy_abs && cudaMemsetAsync(v_xy_abs, 0, n * 2 * sizeof(float), s) != cudaSuccess))
        return check_launch("raster_bwd output memset");
    if (count == 0) return SPLAT_OK;  // lib/ops.cu:184-186
    RasterBwdArgs a;
    a.tiles_x = tiles_x(p); a.width = p.img_width; a.height = p.img_height; a.bw = p.block_width;
    a.n = (int)p.num_points; a.status = p.device_status;
    a.count = count; a.ids = ids; a.bins = bins;
    a.xys = xys; a.conics = conics; a.colors = colors; a.opac = opac; a.background = background;
    a.final_Ts = final_Ts; a.final_idx = final_idx; a.v_img = v_img; a.v_alpha = v_alpha;
    a.v_colors = v_colors; a.v_opac = v_opac; a.v_xy = v_xy; a.v_xy_abs = v_xy_abs;
    a.v_conic = v_conic;
    dim3 grid(tiles_x(p), tiles_y(p)), block(p.block_width, p.block_width);
    if (v_xy_abs)
        raster_bwd_kernel<true><<<grid, block, 0, s>>>(a);
    else
        raster_bwd_kernel<false><<<grid, block, 0, s>>>(a);
    return check_launch("raster_bwd_kernel");
}

}  // namespace splat
