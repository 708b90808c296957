// fit.cu -- the fitting loop's per-Gaussian parameter maps and Adam update.
//
// examples/single_image.py:143-148 renders from raw parameters:
//   quats     = q / |q|            (jnp.linalg.norm over the last axis)
//   colors    = sigmoid(c)
//   opacities = sigmoid(o)
// (means and scales are used as they are) and fits them with
// optax.adam(lr) (b1 = 0.9, b2 = 0.999, eps = 1e-8, eps_root = 0) on the L2
// loss (single_image.py:26-40).  fit_transform_kernel applies the maps;
// fit_adam_kernel takes the render's gradients with respect to the mapped
// parameters, applies the chain rule of the maps and the Adam update to all
// 14 raw parameters of a Gaussian in one pass.
#include "splat_internal.cuh"

namespace splat {

__device__ __forceinline__ float sigmoidf(float x) { return 1.f / (1.f + expf(-x)); }

struct FitTransformArgs {
    int n;
    const float *quats_raw, *colors_raw, *opac_raw;
    float *quats, *colors, *opac;
};

__global__ void fit_transform_kernel(FitTransformArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 q = reinterpret_cast<const float4 *>(a.quats_raw)[i];
    const float inv = rsqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    reinterpret_cast<float4 *>(a.quats)[i] = make_float4(q.x * inv, q.y * inv, q.z * inv, q.w * inv);
#pragma unroll
    for (int k = 0; k < 3; ++k) a.colors[3 * i + k] = sigmoidf(a.colors_raw[3 * i + k]);
    a.opac[i] = sigmoidf(a.opac_raw[i]);
}

struct FitAdamArgs {
    int n;
    float lr, b1, b2, eps;
    const int *step;  // device step counter t (1-based after the update)
    // raw parameters (updated in place) and their Adam moments
    float *means, *scales, *quats_raw, *colors_raw, *opac_raw;
    float *m, *v;  // (N, 14) each: means 3, scales 3, quats 4, colors 3, opacity 1
    // gradients with respect to the mapped parameters
    const float *g_means, *g_scales, *g_quats, *g_colors, *g_opac;
    // the mapped values (for the chain rule)
    const float *quats, *colors, *opac;
};

__device__ __forceinline__ void adam1(float &p, float g, float &m, float &v, float lr, float b1,
                                      float b2, float eps, float c1, float c2) {
    m = b1 * m + (1.f - b1) * g;
    v = b2 * v + (1.f - b2) * g * g;
    const float mh = m / c1;
    const float vh = v / c2;
    p -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void fit_adam_kernel(FitAdamArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int t = *a.step;
    const float c1 = 1.f - powf(a.b1, (float)t);
    const float c2 = 1.f - powf(a.b2, (float)t);
    float g[14];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        g[k] = a.g_means[3 * i + k];
        g[3 + k] = a.g_scales[3 * i + k];
    }
    // d(q/|q|)/dq applied to the cotangent: (v - qn (qn . v)) / |q|
    const float4 qr = reinterpret_cast<const float4 *>(a.quats_raw)[i];
    const float4 qn = reinterpret_cast<const float4 *>(a.quats)[i];
    const float4 vq = reinterpret_cast<const float4 *>(a.g_quats)[i];
    const float inv = rsqrtf(qr.x * qr.x + qr.y * qr.y + qr.z * qr.z + qr.w * qr.w);
    const float dot = qn.x * vq.x + qn.y * vq.y + qn.z * vq.z + qn.w * vq.w;
    g[6] = (vq.x - qn.x * dot) * inv;
    g[7] = (vq.y - qn.y * dot) * inv;
    g[8] = (vq.z - qn.z * dot) * inv;
    g[9] = (vq.w - qn.w * dot) * inv;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float s = a.colors[3 * i + k];
        g[10 + k] = a.g_colors[3 * i + k] * s * (1.f - s);
    }
    const float so = a.opac[i];
    g[13] = a.g_opac[i] * so * (1.f - so);
    float *m = a.m + 14 * (size_t)i, *v = a.v + 14 * (size_t)i;
    float *p[14] = {&a.means[3 * i], &a.means[3 * i + 1], &a.means[3 * i + 2],
                    &a.scales[3 * i], &a.scales[3 * i + 1], &a.scales[3 * i + 2],
                    &a.quats_raw[4 * i], &a.quats_raw[4 * i + 1], &a.quats_raw[4 * i + 2],
                    &a.quats_raw[4 * i + 3], &a.colors_raw[3 * i], &a.colors_raw[3 * i + 1],
                    &a.colors_raw[3 * i + 2], &a.opac_raw[i]};
#pragma unroll
    for (int k = 0; k < 14; ++k) {
        float pk = *p[k], mk = m[k], vk = v[k];
        adam1(pk, g[k], mk, vk, a.lr, a.b1, a.b2, a.eps, c1, c2);
        *p[k] = pk;
        m[k] = mk;
        v[k] = vk;
    }
}

__global__ void fit_step_kernel(int *step) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

}  // namespace splat

using namespace splat;

extern "C" {

int splat_fit_transform(int n, const float *quats_raw, const float *colors_raw,
                        const float *opac_raw, float *quats, float *colors, float *opac,
                        splat_stream_t stream) {
    if (n < 0) return fail(SPLAT_ERR_INVALID_ARG, "n must be non-negative");
    if (n == 0) return SPLAT_OK;
    if (!quats_raw || !colors_raw || !opac_raw || !quats || !colors || !opac)
        return fail(SPLAT_ERR_INVALID_ARG, "a parameter pointer is NULL");
    FitTransformArgs a{n, quats_raw, colors_raw, opac_raw, quats, colors, opac};
    fit_transform_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(a);
    return check_launch("fit_transform_kernel");
}

int splat_fit_adam(int n, float lr, int *step_dev, float *means, float *scales, float *quats_raw,
                   float *colors_raw, float *opac_raw, float *m, float *v, const float *g_means,
                   const float *g_scales, const float *g_quats, const float *g_colors,
                   const float *g_opac, const float *quats, const float *colors,
                   const float *opac, splat_stream_t stream) {
    if (n < 0) return fail(SPLAT_ERR_INVALID_ARG, "n must be non-negative");
    if (!step_dev) return fail(SPLAT_ERR_INVALID_ARG, "step_dev is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    fit_step_kernel<<<1, 32, 0, s>>>(step_dev);
    if (int rc = check_launch("fit_step_kernel")) return rc;
    if (n == 0) return SPLAT_OK;
    FitAdamArgs a;
    a.n = n;
    a.lr = lr;
    a.b1 = 0.9f;
    a.b2 = 0.999f;
    a.eps = 1e-8f;
    a.step = step_dev;
    a.means = means; a.scales = scales; a.quats_raw = quats_raw;
    a.colors_raw = colors_raw; a.opac_raw = opac_raw;
    a.m = m; a.v = v;
    a.g_means = g_means; a.g_scales = g_scales; a.g_quats = g_quats;
    a.g_colors = g_colors; a.g_opac = g_opac;
    a.quats = quats; a.colors = colors; a.opac = opac;
    fit_adam_kernel<<<(n + 255) / 256, 256, 0, s>>>(a);
    return check_launch("fit_adam_kernel");
}

}  // extern "C"
