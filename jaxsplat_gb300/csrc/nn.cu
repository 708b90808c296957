// nn.cu -- the warm-start network's non-GEMM kernels: 3x3 convolutions as
// im2col + tensor-core GEMM (gemm_tc.cu), so this file holds the gathers
// around the GEMM (im2col, col2im), the bias/ReLU epilogue and its gradient,
// and the Adam update.  Activations are NHWC bf16,
// gradients fp32, weights fp32 masters with bf16 copies for the GEMMs.
#include <cuda_bf16.h>

#include <algorithm>

#include "splat_internal.cuh"

namespace splat {

// cols[p, (ky*3 + kx)*C + c] = x[n, oy*s + ky - 1, ox*s + kx - 1, c] (zero
// outside), p = (n*Ho + oy)*Wo + ox; columns past 9C up to kpad are zero.
// One thread per 8-column chunk of a row of cols (kpad a multiple of 8, cols
// 16-byte aligned), one block row per output row (b, oy), 32-bit index
// arithmetic: consecutive threads write consecutive 16-byte chunks.  kVec:
// C a multiple of 8 and x 16-byte aligned, so a chunk is 8 channels of one
// tap, read as one 16-byte load.
template <bool kVec, int kC = 0>
__global__ void im2col3x3_kernel(const __nv_bfloat16 *x, __nv_bfloat16 *cols, int n, int h, int w,
                                 int c_rt, int stride, int ho, int wo, int kpad_rt) {
    // kC > 0: C (and kpad = 9C) fixed at compile time, the index splits are
    // shifts and multiplies
    const int c = kC > 0 ? kC : c_rt;
    const int kpad = kC > 0 ? 9 * kC : kpad_rt;
    const int nch = kpad >> 3;
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= wo * nch) return;
    const int ox = item / nch, j = item - ox * nch;
    for (int row = blockIdx.y; row < n * ho; row += gridDim.y) {
        const int b = row / ho, oy = row - b * ho;
        const size_t p = (size_t)row * wo + ox;
        uint4 out = make_uint4(0u, 0u, 0u, 0u);
        const int k0 = j << 3;
        if (kVec) {
            if (k0 < 9 * c) {
                const int tap = k0 / c, ch = k0 - tap * c;
                const int iy = oy * stride + tap / 3 - 1, ix = ox * stride + tap % 3 - 1;
                if (iy >= 0 && iy < h && ix >= 0 && ix < w)
                    out = *reinterpret_cast<const uint4 *>(x + ((size_t)(b * h + iy) * w + ix) * c + ch);
            }
        } else {
            uint32_t word[4] = {0u, 0u, 0u, 0u};
            int tap = k0 / c, ch = k0 - tap * c;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (tap < 9) {
                    const int iy = oy * stride + tap / 3 - 1, ix = ox * stride + tap % 3 - 1;
                    if (iy >= 0 && iy < h && ix >= 0 && ix < w) {
                        const uint32_t bits = __bfloat16_as_ushort(
                            x[((size_t)(b * h + iy) * w + ix) * c + ch]);
                        word[q >> 1] |= bits << ((q & 1) * 16);
                    }
                }
                if (++ch == c) {
                    ch = 0;
                    ++tap;
                }
            }
            out = make_uint4(word[0], word[1], word[2], word[3]);
        }
        *reinterpret_cast<uint4 *>(cols + p * kpad + k0) = out;
    }
}

// im2col for few channels (C not a multiple of 8, e.g. the RGB input): one
// block per output row (b, oy) stages the three input rows it reads in
// shared memory with 16-byte loads, then each thread assembles an output
// pixel's kpad columns from there and writes them as 16-byte chunks.  The
// three rows take 3 * w * C bf16 of shared memory (w * C <= 8192).  kC > 0
// fixes C at compile time (the column -> (tap, channel) split is then a
// multiply instead of a division per element).
template <int kC>
__global__ void im2col3x3_rows_kernel(const __nv_bfloat16 *__restrict__ x,
                                      __nv_bfloat16 *__restrict__ cols, int n, int h, int w,
                                      int c_rt, int stride, int ho, int wo, int kpad_rt) {
    const int c = kC > 0 ? kC : c_rt;
    // kC > 0: kpad = 9C rounded up to 8, so the column loop unrolls fully
    const int kpad = kC > 0 ? (9 * kC + 7) / 8 * 8 : kpad_rt;
    extern __shared__ __align__(16) uint8_t s_rows_raw[];
    __nv_bfloat16 *s_rows = reinterpret_cast<__nv_bfloat16 *>(s_rows_raw);
    const int rowlen = w * c;  // bf16 per input row
    for (int row = blockIdx.x; row < n * ho; row += gridDim.x) {
        const int b = row / ho, oy = row - b * ho;
        __syncthreads();  // the previous row's readers are done
        for (int ky = 0; ky < 3; ++ky) {
            const int iy = oy * stride + ky - 1;
            __nv_bfloat16 *dst = s_rows + ky * rowlen;
            if (iy < 0 || iy >= h) {
                for (int e = threadIdx.x; e < rowlen; e += blockDim.x) dst[e] = __float2bfloat16(0.f);
                continue;
            }
            const __nv_bfloat16 *src = x + (size_t)(b * h + iy) * rowlen;
            if (((reinterpret_cast<uintptr_t>(src)) & 15u) == 0 && (rowlen & 7) == 0) {
                for (int e = threadIdx.x; e < rowlen / 8; e += blockDim.x)
                    reinterpret_cast<uint4 *>(dst)[e] = __ldg(reinterpret_cast<const uint4 *>(src) + e);
            } else {
                for (int e = threadIdx.x; e < rowlen; e += blockDim.x) dst[e] = src[e];
            }
        }
        __syncthreads();
        for (int ox = threadIdx.x; ox < wo; ox += blockDim.x) {
            __nv_bfloat16 *out = cols + ((size_t)row * wo + ox) * kpad;
#pragma unroll
            for (int k0 = 0; k0 < kpad; k0 += 8) {
                uint32_t word[4] = {0u, 0u, 0u, 0u};
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k = k0 + q;
                    if (k < 9 * c) {
                        const int tap = k / c, ch = k - tap * c;
                        const int ix = ox * stride + tap % 3 - 1;
                        if (ix >= 0 && ix < w) {
                            const uint32_t bits =
                                __bfloat16_as_ushort(s_rows[(tap / 3) * rowlen + ix * c + ch]);
                            word[q >> 1] |= bits << ((q & 1) * 16);
                        }
                    }
                }
                *reinterpret_cast<uint4 *>(out + k0) = make_uint4(word[0], word[1], word[2], word[3]);
            }
        }
    }
}

// dx[n, iy, ix, c] = sum over the (output pixel, tap) pairs that read it of
// dcols[p, tap*C + c] (a gather, so no atomics; taps summed ky-major).
// One thread per 4 channels of an input pixel (C and kpad multiples of 4,
// both buffers 16-byte aligned): float4 loads and stores, one block row per
// input row (b, iy), 32-bit index arithmetic.
__global__ void col2im3x3_kernel(const float *dcols, float *dx, int n, int h, int w, int c,
                                 int stride, int ho, int wo, int kpad) {
    const int c4 = c >> 2;
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= w * c4) return;
    const int ix = item / c4, ch = (item - ix * c4) << 2;
    for (int row = blockIdx.y; row < n * h; row += gridDim.y) {
        const int b = row / h, iy = row - b * h;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int ky = 0; ky < 3; ++ky) {
            const int ty = iy + 1 - ky;
            if (ty < 0 || ty % stride) continue;
            const int oy = ty / stride;
            if (oy >= ho) continue;
#pragma unroll
            for (int kx = 0; kx < 3; ++kx) {
                const int tx = ix + 1 - kx;
                if (tx < 0 || tx % stride) continue;
                const int ox = tx / stride;
                if (ox >= wo) continue;
                const size_t p = (size_t)(b * ho + oy) * wo + ox;
                const float4 d =
                    *reinterpret_cast<const float4 *>(dcols + p * kpad + (ky * 3 + kx) * c + ch);
                acc.x += d.x;
                acc.y += d.y;
                acc.z += d.z;
                acc.w += d.w;
            }
        }
        *reinterpret_cast<float4 *>(dx + ((size_t)row * w + ix) * c + ch) = acc;
    }
}

// The same gather one element per thread, for C or kpad not a multiple of 4.
__global__ void col2im3x3_scalar_kernel(const float *dcols, float *dx, int n, int h, int w, int c,
                                        int stride, int ho, int wo, int kpad) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= w * c) return;
    const int ix = item / c, ch = item - ix * c;
    for (int row = blockIdx.y; row < n * h; row += gridDim.y) {
        const int b = row / h, iy = row - b * h;
        float acc = 0.f;
#pragma unroll
        for (int ky = 0; ky < 3; ++ky) {
            const int ty = iy + 1 - ky;
            if (ty < 0 || ty % stride) continue;
            const int oy = ty / stride;
            if (oy >= ho) continue;
#pragma unroll
            for (int kx = 0; kx < 3; ++kx) {
                const int tx = ix + 1 - kx;
                if (tx < 0 || tx % stride) continue;
                const int ox = tx / stride;
                if (ox >= wo) continue;
                const size_t p = (size_t)(b * ho + oy) * wo + ox;
                acc += dcols[p * kpad + (ky * 3 + kx) * c + ch];
            }
        }
        dx[((size_t)row * w + ix) * c + ch] = acc;
    }
}

// col2im fused with the gradient through the previous layer's ReLU: the
// gathered sum dx (the same taps in the same order as col2im3x3_kernel) is
// masked by y > 0 (y: the previous layer's bf16 output, NHWC like dx) and
// written as bf16 dz, and dz's channel sums are added into dbias -- so the
// fp32 dx is never stored and re-read.  Four channels per thread (C and kpad
// multiples of 4, dcols 16-byte and y, dz 8-byte aligned); a thread keeps
// its channels over the rows it walks and sums them in registers.
__global__ void col2im_act3x3_kernel(const float *dcols, const __nv_bfloat16 *y,
                                     __nv_bfloat16 *dz, float *dbias, int n, int h, int w, int c,
                                     int stride, int ho, int wo, int kpad) {
    extern __shared__ float s_db[];
    for (int j = threadIdx.x; j < c; j += blockDim.x) s_db[j] = 0.f;
    __syncthreads();
    const int c4 = c >> 2;
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = item / c4, ch = (item - ix * c4) << 2;
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    if (item < w * c4) {
        for (int row = blockIdx.y; row < n * h; row += gridDim.y) {
            const int b = row / h, iy = row - b * h;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int ky = 0; ky < 3; ++ky) {
                const int ty = iy + 1 - ky;
                if (ty < 0 || ty % stride) continue;
                const int oy = ty / stride;
                if (oy >= ho) continue;
#pragma unroll
                for (int kx = 0; kx < 3; ++kx) {
                    const int tx = ix + 1 - kx;
                    if (tx < 0 || tx % stride) continue;
                    const int ox = tx / stride;
                    if (ox >= wo) continue;
                    const size_t p = (size_t)(b * ho + oy) * wo + ox;
                    const float4 d = *reinterpret_cast<const float4 *>(dcols + p * kpad +
                                                                       (ky * 3 + kx) * c + ch);
                    acc.x += d.x;
                    acc.y += d.y;
                    acc.z += d.z;
                    acc.w += d.w;
                }
            }
            const size_t o = ((size_t)row * w + ix) * c + ch;
            const uint2 yb = *reinterpret_cast<const uint2 *>(y + o);
            const __nv_bfloat162 y01 = *reinterpret_cast<const __nv_bfloat162 *>(&yb.x);
            const __nv_bfloat162 y23 = *reinterpret_cast<const __nv_bfloat162 *>(&yb.y);
            if (!(__low2float(y01) > 0.f)) acc.x = 0.f;
            if (!(__high2float(y01) > 0.f)) acc.y = 0.f;
            if (!(__low2float(y23) > 0.f)) acc.z = 0.f;
            if (!(__high2float(y23) > 0.f)) acc.w = 0.f;
            const __nv_bfloat162 d01 = __floats2bfloat162_rn(acc.x, acc.y);
            const __nv_bfloat162 d23 = __floats2bfloat162_rn(acc.z, acc.w);
            uint2 out;
            out.x = *reinterpret_cast<const uint32_t *>(&d01);
            out.y = *reinterpret_cast<const uint32_t *>(&d23);
            *reinterpret_cast<uint2 *>(dz + o) = out;
            sum.x += acc.x;
            sum.y += acc.y;
            sum.z += acc.z;
            sum.w += acc.w;
        }
        atomicAdd(&s_db[ch], sum.x);
        atomicAdd(&s_db[ch + 1], sum.y);
        atomicAdd(&s_db[ch + 2], sum.z);
        atomicAdd(&s_db[ch + 3], sum.w);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < c; j += blockDim.x)
        if (s_db[j] != 0.f) atomicAdd(&dbias[j], s_db[j]);
}

// The stride-2 form of col2im_act3x3_kernel: one thread per 4 channels of a
// 2x2 quad of input pixels (2m + dy, 2n + dx), whose taps are exactly the 9
// taps of output pixels (m, n), (m, n+1), (m+1, n), (m+1, n+1) -- all nine
// 16-byte loads in flight at once; each pixel's taps summed in the same
// (ky, kx) order as col2im3x3_kernel, so dz is bit-identical to col2im
// followed by act_grad.  256 / (c / 4) threads per block share a channel
// group along the grid-stride walk (c / 4 divides 256).
__global__ void col2im_act3x3_s2_kernel(const float *__restrict__ dcols,
                                        const __nv_bfloat16 *__restrict__ y,
                                        __nv_bfloat16 *__restrict__ dz, float *__restrict__ dbias,
                                        int n, int h, int w, int c, int ho, int wo, int kpad) {
    extern __shared__ float s_db[];
    for (int j = threadIdx.x; j < c; j += blockDim.x) s_db[j] = 0.f;
    __syncthreads();
    const int c4 = c >> 2, hq = (h + 1) >> 1, wq = (w + 1) >> 1;
    const int total = n * hq * wq * c4;
    const int stride = gridDim.x * blockDim.x;
    int item = blockIdx.x * blockDim.x + threadIdx.x;
    const int ch = (item % c4) << 2;  // fixed: stride is a multiple of c4
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    for (; item < total; item += stride) {
        const int q = item / c4;
        const int nq = q % wq, r = q / wq;
        const int mq = r % hq, b = r / hq;
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                const int iy = 2 * mq + dy, ix = 2 * nq + dx;
                if (iy >= h || ix >= w) continue;
                float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int ky = 0; ky < 3; ++ky) {
                    // ty = iy + 1 - ky must be even: ky = 1 for even rows,
                    // ky = 0 (oy = mq + 1) and 2 (oy = mq) for odd rows
                    if ((dy + 1 - ky) & 1) continue;
                    const int oy = (iy + 1 - ky) >> 1;
                    if (oy < 0 || oy >= ho) continue;
#pragma unroll
                    for (int kx = 0; kx < 3; ++kx) {
                        if ((dx + 1 - kx) & 1) continue;
                        const int ox = (ix + 1 - kx) >> 1;
                        if (ox < 0 || ox >= wo) continue;
                        const size_t p = (size_t)(b * ho + oy) * wo + ox;
                        const float4 d = __ldg(reinterpret_cast<const float4 *>(
                            dcols + p * kpad + (ky * 3 + kx) * c + ch));
                        acc.x += d.x;
                        acc.y += d.y;
                        acc.z += d.z;
                        acc.w += d.w;
                    }
                }
                const size_t o = ((size_t)(b * h + iy) * w + ix) * c + ch;
                const uint2 yb = __ldg(reinterpret_cast<const uint2 *>(y + o));
                const __nv_bfloat162 y01 = *reinterpret_cast<const __nv_bfloat162 *>(&yb.x);
                const __nv_bfloat162 y23 = *reinterpret_cast<const __nv_bfloat162 *>(&yb.y);
                if (!(__low2float(y01) > 0.f)) acc.x = 0.f;
                if (!(__high2float(y01) > 0.f)) acc.y = 0.f;
                if (!(__low2float(y23) > 0.f)) acc.z = 0.f;
                if (!(__high2float(y23) > 0.f)) acc.w = 0.f;
                const __nv_bfloat162 d01 = __floats2bfloat162_rn(acc.x, acc.y);
                const __nv_bfloat162 d23 = __floats2bfloat162_rn(acc.z, acc.w);
                uint2 out;
                out.x = *reinterpret_cast<const uint32_t *>(&d01);
                out.y = *reinterpret_cast<const uint32_t *>(&d23);
                *reinterpret_cast<uint2 *>(dz + o) = out;
                sum.x += acc.x;
                sum.y += acc.y;
                sum.z += acc.z;
                sum.w += acc.w;
            }
        }
    }
    if (blockIdx.x * blockDim.x + threadIdx.x < total) {
        atomicAdd(&s_db[ch], sum.x);
        atomicAdd(&s_db[ch + 1], sum.y);
        atomicAdd(&s_db[ch + 2], sum.z);
        atomicAdd(&s_db[ch + 3], sum.w);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < c; j += blockDim.x)
        if (s_db[j] != 0.f) atomicAdd(&dbias[j], s_db[j]);
}

// y = act(acc + bias) as bf16 (act: ReLU when relu != 0); rows x cols.
__global__ void bias_act_kernel(const float *acc, const float *bias, __nv_bfloat16 *y,
                                float *y32, long long rows, int cols, int relu) {
    const long long total = rows * cols;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        float v = acc[i] + bias[i % cols];
        if (relu) v = fmaxf(v, 0.f);
        if (y) y[i] = __float2bfloat16(v);
        if (y32) y32[i] = v;
    }
}

// Gradient through ReLU (mask from the bf16 output y > 0 when relu != 0):
// dz = dy * [y > 0] written as bf16 (the next GEMMs' operand), and the
// column sums of dz accumulated into dbias.  When cols divides the block
// (a whole number of rows per block) every thread keeps one column and sums
// it in a register; otherwise the column is tracked incrementally along the
// grid-stride loop and summed in shared memory.
__global__ void act_grad_kernel(const float *__restrict__ dy, const __nv_bfloat16 *__restrict__ y,
                                __nv_bfloat16 *__restrict__ dz, float *__restrict__ dbias,
                                long long rows, int cols, int relu) {
    extern __shared__ float s_db[];
    for (int j = threadIdx.x; j < cols; j += blockDim.x) s_db[j] = 0.f;
    __syncthreads();
    const long long total = rows * cols;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (blockDim.x % cols == 0) {
        float sum = 0.f;
#pragma unroll 4
        for (; i < total; i += stride) {
            float g = dy[i];
            if (relu && !(__bfloat162float(y[i]) > 0.f)) g = 0.f;
            dz[i] = __float2bfloat16(g);
            sum += g;
        }
        atomicAdd(&s_db[threadIdx.x % cols], sum);
    } else {
        int col = (int)(i % cols);
        const int step = (int)(stride % cols);
        for (; i < total; i += stride) {
            float g = dy[i];
            if (relu && !(__bfloat162float(y[i]) > 0.f)) g = 0.f;
            dz[i] = __float2bfloat16(g);
            atomicAdd(&s_db[col], g);
            col += step;
            if (col >= cols) col -= cols;
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < cols; j += blockDim.x)
        if (s_db[j] != 0.f) atomicAdd(&dbias[j], s_db[j]);
}

// Adam (b1 0.9, b2 0.999, eps 1e-8) on fp32 masters; refreshes bf16 copies.
__global__ void adam_kernel(float *w, float *m, float *v, const float *g, __nv_bfloat16 *w16,
                            long long n, float lr, float c1, float c2) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = 0.9f * m[i] + 0.1f * gi;
        const float vi = 0.999f * v[i] + 0.001f * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
        w[i] = wi;
        if (w16) w16[i] = __float2bfloat16(wi);
    }
}

// Adam over several parameter arrays in one launch: segment k covers flat
// indices [start[k], start[k+1]); the arithmetic is adam_kernel's.
constexpr int kAdamMaxSegs = 16;
struct AdamSegs {
    float *w[kAdamMaxSegs], *m[kAdamMaxSegs], *v[kAdamMaxSegs];
    const float *g[kAdamMaxSegs];
    __nv_bfloat16 *w16[kAdamMaxSegs];
    long long start[kAdamMaxSegs + 1];
};

__global__ void adam_multi_kernel(AdamSegs a, int nseg, float lr, float c1, float c2) {
    const long long total = a.start[nseg];
    int k = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        while (i >= a.start[k + 1]) ++k;  // i only grows along a thread's walk
        const long long j = i - a.start[k];
        const float gi = a.g[k][j];
        const float mi = 0.9f * a.m[k][j] + 0.1f * gi;
        const float vi = 0.999f * a.v[k][j] + 0.001f * gi * gi;
        a.m[k][j] = mi;
        a.v[k][j] = vi;
        const float wi = a.w[k][j] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
        a.w[k][j] = wi;
        if (a.w16[k]) a.w16[k][j] = __float2bfloat16(wi);
    }
}

static unsigned grid_for(long long total) {
    const long long b = (total + 255) / 256;
    return (unsigned)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

}  // namespace splat

using namespace splat;

extern "C" {

int splat_nn_im2col3x3(const void *x, void *cols, int n, int h, int w, int c, int stride, int kpad,
                       splat_stream_t stream) {
    if (!x || !cols || n <= 0 || h <= 0 || w <= 0 || c <= 0 || (stride != 1 && stride != 2) ||
        kpad < 9 * c || kpad % 8 != 0 || (reinterpret_cast<uintptr_t>(cols) & 15u) ||
        (long long)n * h * w * c >= (1ll << 31))
        return fail(SPLAT_ERR_INVALID_ARG, "im2col3x3: bad arguments");
    const int ho = (h - 1) / stride + 1, wo = (w - 1) / stride + 1;
    const int items = wo * (kpad / 8);
    const dim3 grid((unsigned)((items + 255) / 256), (unsigned)std::min(n * ho, 65535));
    const bool vec = c % 8 == 0 && (reinterpret_cast<uintptr_t>(x) & 15u) == 0;
    const auto *xb = static_cast<const __nv_bfloat16 *>(x);
    auto *cb = static_cast<__nv_bfloat16 *>(cols);
    if (!vec && w * c <= 8192) {
        const int rows = n * ho;
        const unsigned blocks = (unsigned)std::min(rows, 152 * 16);
        const size_t smem = 3 * (size_t)w * c * sizeof(__nv_bfloat16);
        if (c == 3 && kpad == 32)
            im2col3x3_rows_kernel<3><<<blocks, 256, smem, (cudaStream_t)stream>>>(
                xb, cb, n, h, w, c, stride, ho, wo, kpad);
        else
            im2col3x3_rows_kernel<0><<<blocks, 256, smem, (cudaStream_t)stream>>>(
                xb, cb, n, h, w, c, stride, ho, wo, kpad);
        return check_launch("im2col3x3_rows_kernel");
    }
    if (vec && kpad == 9 * c && (c == 32 || c == 64 || c == 128)) {
        auto kern = c == 32 ? im2col3x3_kernel<true, 32>
                            : (c == 64 ? im2col3x3_kernel<true, 64> : im2col3x3_kernel<true, 128>);
        kern<<<grid, 256, 0, (cudaStream_t)stream>>>(xb, cb, n, h, w, c, stride, ho, wo, kpad);
    } else if (vec)
        im2col3x3_kernel<true><<<grid, 256, 0, (cudaStream_t)stream>>>(xb, cb, n, h, w, c, stride,
                                                                       ho, wo, kpad);
    else
        im2col3x3_kernel<false><<<grid, 256, 0, (cudaStream_t)stream>>>(xb, cb, n, h, w, c, stride,
                                                                        ho, wo, kpad);
    return check_launch("im2col3x3_kernel");
}

int splat_nn_col2im3x3(const float *dcols, float *dx, int n, int h, int w, int c, int stride,
                       int kpad, splat_stream_t stream) {
    if (!dcols || !dx || n <= 0 || h <= 0 || w <= 0 || c <= 0 || (stride != 1 && stride != 2) ||
        kpad < 9 * c || (long long)n * h * w * c >= (1ll << 31))
        return fail(SPLAT_ERR_INVALID_ARG, "col2im3x3: bad arguments");
    const int ho = (h - 1) / stride + 1, wo = (w - 1) / stride + 1;
    const unsigned rows = (unsigned)std::min(n * h, 65535);
    const bool vec = c % 4 == 0 && kpad % 4 == 0 &&
                     ((reinterpret_cast<uintptr_t>(dcols) | reinterpret_cast<uintptr_t>(dx)) & 15u) == 0;
    if (vec)
        col2im3x3_kernel<<<dim3((unsigned)((w * (c / 4) + 255) / 256), rows), 256, 0,
                           (cudaStream_t)stream>>>(dcols, dx, n, h, w, c, stride, ho, wo, kpad);
    else
        col2im3x3_scalar_kernel<<<dim3((unsigned)((w * c + 255) / 256), rows), 256, 0,
                                  (cudaStream_t)stream>>>(dcols, dx, n, h, w, c, stride, ho, wo,
                                                          kpad);
    return check_launch("col2im3x3_kernel");
}

int splat_nn_col2im_act3x3(const float *dcols, const void *y, void *dz, float *dbias, int n,
                           int h, int w, int c, int stride, int kpad, splat_stream_t stream) {
    if (!dcols || !y || !dz || !dbias || n <= 0 || h <= 0 || w <= 0 || c <= 0 || c % 4 ||
        c > 4096 || kpad % 4 || (stride != 1 && stride != 2) || kpad < 9 * c ||
        (long long)n * h * w * c >= (1ll << 31) ||
        (reinterpret_cast<uintptr_t>(dcols) & 15u) ||
        ((reinterpret_cast<uintptr_t>(y) | reinterpret_cast<uintptr_t>(dz)) & 7u))
        return fail(SPLAT_ERR_INVALID_ARG, "col2im_act3x3: bad arguments");
    const int ho = (h - 1) / stride + 1, wo = (w - 1) / stride + 1;
    if (stride == 2 && 256 % (c / 4) == 0) {
        const long long quads = (long long)n * ((h + 1) / 2) * ((w + 1) / 2) * (c / 4);
        // one wave of resident blocks, each thread walking several quads
        int dev = 0, sms = 152, per_sm = 4;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, col2im_act3x3_s2_kernel, 256,
                                                      c * sizeof(float));
        const long long wave = (long long)std::max(1, sms) * std::max(1, per_sm);
        const unsigned blocks = (unsigned)std::max(1ll, std::min((quads + 255) / 256, wave));
        col2im_act3x3_s2_kernel<<<blocks, 256, c * sizeof(float), (cudaStream_t)stream>>>(
            dcols, static_cast<const __nv_bfloat16 *>(y), static_cast<__nv_bfloat16 *>(dz), dbias,
            n, h, w, c, ho, wo, kpad);
        return check_launch("col2im_act3x3_s2_kernel");
    }
    // ~8 blocks per SM; each thread walks several rows, so the channel sums
    // reach global memory from few blocks
    const unsigned gx = (unsigned)((w * (c / 4) + 255) / 256);
    const unsigned rows = (unsigned)std::max(1, std::min(n * h, (int)(152 * 8 / gx)));
    col2im_act3x3_kernel<<<dim3(gx, rows), 256,
                           c * sizeof(float), (cudaStream_t)stream>>>(
        dcols, static_cast<const __nv_bfloat16 *>(y), static_cast<__nv_bfloat16 *>(dz), dbias, n,
        h, w, c, stride, ho, wo, kpad);
    return check_launch("col2im_act3x3_kernel");
}

int splat_nn_bias_act(const float *acc, const float *bias, void *y, float *y32, int64_t rows,
                      int cols, int relu, splat_stream_t stream) {
    if (!acc || !bias || (!y && !y32) || rows < 0 || cols <= 0)
        return fail(SPLAT_ERR_INVALID_ARG, "bias_act: bad arguments");
    bias_act_kernel<<<grid_for(rows * cols), 256, 0, (cudaStream_t)stream>>>(
        acc, bias, static_cast<__nv_bfloat16 *>(y), y32, rows, cols, relu);
    return check_launch("bias_act_kernel");
}

int splat_nn_act_grad(const float *dy, const void *y, void *dz, float *dbias, int64_t rows,
                      int cols, int relu, splat_stream_t stream) {
    if (!dy || !dz || !dbias || (relu && !y) || rows < 0 || cols <= 0 || cols > 4096)
        return fail(SPLAT_ERR_INVALID_ARG, "act_grad: bad arguments");
    // a block of a whole number of rows when cols is a multiple of 32 (every
    // thread keeps one column); about two blocks per SM, so few blocks add
    // their column sums into dbias
    const int threads = (cols % 32 == 0 && cols <= 1024) ? cols * std::max(1, 256 / cols) : 256;
    const long long blocks =
        std::max(1ll, std::min((long long)((rows * cols + threads - 1) / threads), 304ll));
    act_grad_kernel<<<(unsigned)blocks, threads, cols * sizeof(float), (cudaStream_t)stream>>>(
        dy, static_cast<const __nv_bfloat16 *>(y), static_cast<__nv_bfloat16 *>(dz), dbias, rows,
        cols, relu);
    return check_launch("act_grad_kernel");
}

int splat_nn_adam(float *w, float *m, float *v, const float *g, void *w16, int64_t n, float lr,
                  int step, splat_stream_t stream) {
    if (!w || !m || !v || !g || n < 0 || step < 1)
        return fail(SPLAT_ERR_INVALID_ARG, "adam: bad arguments");
    const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
    adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(
        w, m, v, g, static_cast<__nv_bfloat16 *>(w16), n, lr, c1, c2);
    return check_launch("adam_kernel");
}

int splat_nn_adam_multi(const splat_adam_seg *segs, int nseg, float lr, int step,
                        splat_stream_t stream) {
    if (!segs || nseg <= 0 || nseg > kAdamMaxSegs || step < 1)
        return fail(SPLAT_ERR_INVALID_ARG, "adam_multi: bad arguments");
    AdamSegs a{};
    a.start[0] = 0;
    for (int k = 0; k < nseg; ++k) {
        const splat_adam_seg &sg = segs[k];
        if (sg.n < 0 || (sg.n > 0 && (!sg.w || !sg.m || !sg.v || !sg.g)))
            return fail(SPLAT_ERR_INVALID_ARG, "adam_multi: bad segment %d", k);
        a.w[k] = sg.w;
        a.m[k] = sg.m;
        a.v[k] = sg.v;
        a.g[k] = sg.g;
        a.w16[k] = static_cast<__nv_bfloat16 *>(sg.w16);
        a.start[k + 1] = a.start[k] + sg.n;
    }
    for (int k = nseg + 1; k <= kAdamMaxSegs; ++k) a.start[k] = a.start[nseg];
    const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
    adam_multi_kernel<<<grid_for(a.start[nseg]), 256, 0, (cudaStream_t)stream>>>(a, nseg, lr, c1,
                                                                                   c2);
    return check_launch("adam_multi_kernel");
}

}  // extern "C"
