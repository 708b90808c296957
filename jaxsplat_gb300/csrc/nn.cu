// nn.cu -- the warm-start network's non-GEMM kernels: 3x3 convolutions as
// im2col + tensor-core GEMM (gemm_tc.cu), so this file holds the gathers
// around the GEMM (im2col, col2im), the bias/ReLU epilogue and its gradient,
// operand transposes and the Adam update.  Activations are NHWC bf16,
// gradients fp32, weights fp32 masters with bf16 copies for the GEMMs.
#include <cuda_bf16.h>

#include "splat_internal.cuh"

namespace splat {

// cols[p, (ky*3 + kx)*C + c] = x[n, oy*s + ky - 1, ox*s + kx - 1, c] (zero
// outside), p = (n*Ho + oy)*Wo + ox; columns past 9C up to kpad are zero.
__global__ void im2col3x3_kernel(const __nv_bfloat16 *x, __nv_bfloat16 *cols, int n, int h, int w,
                                 int c, int stride, int ho, int wo, int kpad) {
    const long long total = (long long)n * ho * wo * kpad;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i % kpad);
        const long long p = i / kpad;
        __nv_bfloat16 v = __float2bfloat16(0.f);
        if (k < 9 * c) {
            const int tap = k / c, ch = k % c;
            const int ox = (int)(p % wo), oy = (int)((p / wo) % ho), b = (int)(p / ((long long)wo * ho));
            const int iy = oy * stride + tap / 3 - 1, ix = ox * stride + tap % 3 - 1;
            if (iy >= 0 && iy < h && ix >= 0 && ix < w)
                v = x[(((size_t)b * h + iy) * w + ix) * c + ch];
        }
        cols[i] = v;
    }
}

// dx[n, iy, ix, c] = sum over the (output pixel, tap) pairs that read it of
// dcols[p, tap*C + c] (a gather, so no atomics).
__global__ void col2im3x3_kernel(const float *dcols, float *dx, int n, int h, int w, int c,
                                 int stride, int ho, int wo, int kpad) {
    const long long total = (long long)n * h * w * c;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const int ix = (int)((i / c) % w), iy = (int)((i / ((long long)c * w)) % h);
        const int b = (int)(i / ((long long)c * w * h));
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
                const size_t p = ((size_t)b * ho + oy) * wo + ox;
                acc += dcols[p * kpad + (ky * 3 + kx) * c + ch];
            }
        }
        dx[i] = acc;
    }
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
// column sums of dz accumulated into dbias.
__global__ void act_grad_kernel(const float *dy, const __nv_bfloat16 *y, __nv_bfloat16 *dz,
                                float *dbias, long long rows, int cols, int relu) {
    extern __shared__ float s_db[];
    for (int j = threadIdx.x; j < cols; j += blockDim.x) s_db[j] = 0.f;
    __syncthreads();
    const long long total = rows * cols;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        float g = dy[i];
        if (relu && !(__bfloat162float(y[i]) > 0.f)) g = 0.f;
        dz[i] = __float2bfloat16(g);
        atomicAdd(&s_db[i % cols], g);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < cols; j += blockDim.x)
        if (s_db[j] != 0.f) atomicAdd(&dbias[j], s_db[j]);
}

// out[c, r] = in[r, c] for a rows x cols bf16 matrix (32x32 tiles).
__global__ void transpose_bf16_kernel(const __nv_bfloat16 *in, __nv_bfloat16 *out, long long rows,
                                      int cols, long long ld_out) {
    __shared__ __nv_bfloat16 tile[32][33];
    const long long r0 = (long long)blockIdx.y * 32;
    const int c0 = blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const long long r = r0 + k;
        const int c = c0 + threadIdx.x;
        tile[k][threadIdx.x] = (r < rows && c < cols) ? in[r * cols + c] : __float2bfloat16(0.f);
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k;
        const long long r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(long long)c * ld_out + r] = tile[threadIdx.x][k];
    }
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
        kpad < 9 * c)
        return fail(SPLAT_ERR_INVALID_ARG, "im2col3x3: bad arguments");
    const int ho = (h - 1) / stride + 1, wo = (w - 1) / stride + 1;
    const long long total = (long long)n * ho * wo * kpad;
    im2col3x3_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const __nv_bfloat16 *>(x), static_cast<__nv_bfloat16 *>(cols), n, h, w, c,
        stride, ho, wo, kpad);
    return check_launch("im2col3x3_kernel");
}

int splat_nn_col2im3x3(const float *dcols, float *dx, int n, int h, int w, int c, int stride,
                       int kpad, splat_stream_t stream) {
    if (!dcols || !dx || n <= 0 || h <= 0 || w <= 0 || c <= 0 || (stride != 1 && stride != 2) ||
        kpad < 9 * c)
        return fail(SPLAT_ERR_INVALID_ARG, "col2im3x3: bad arguments");
    const int ho = (h - 1) / stride + 1, wo = (w - 1) / stride + 1;
    const long long total = (long long)n * h * w * c;
    col2im3x3_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(dcols, dx, n, h, w, c,
                                                                         stride, ho, wo, kpad);
    return check_launch("col2im3x3_kernel");
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
    act_grad_kernel<<<grid_for(rows * cols), 256, cols * sizeof(float), (cudaStream_t)stream>>>(
        dy, static_cast<const __nv_bfloat16 *>(y), static_cast<__nv_bfloat16 *>(dz), dbias, rows,
        cols, relu);
    return check_launch("act_grad_kernel");
}

int splat_nn_transpose_bf16(const void *in, void *out, int64_t rows, int cols, int64_t ld_out,
                            splat_stream_t stream) {
    if (!in || !out || rows < 0 || cols <= 0 || ld_out < rows)
        return fail(SPLAT_ERR_INVALID_ARG, "transpose_bf16: bad arguments");
    dim3 grid((cols + 31) / 32, (unsigned)((rows + 31) / 32));
    if (grid.y > 65535) return fail(SPLAT_ERR_INVALID_ARG, "transpose_bf16: too many rows");
    transpose_bf16_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(
        static_cast<const __nv_bfloat16 *>(in), static_cast<__nv_bfloat16 *>(out), rows, cols,
        ld_out);
    return check_launch("transpose_bf16_kernel");
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

}  // extern "C"
