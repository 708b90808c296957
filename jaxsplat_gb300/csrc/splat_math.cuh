// splat_math.cuh -- device math shared by the projection and raster kernels.
//
// The floating-point expressions below are written in the same algebraic
// form and evaluation order as the reference's (lib/kernels/helpers.h,
// lib/kernels/forward.cu, lib/kernels/backward.cu, lib/common.h), because the
// intersection keys, tile counts and final_idx are integer outputs decided by
// float comparisons: nvcc contracts a*b+c into one FMA according to how the
// expression is written, so the same expression shapes give the same bits.
// The code itself is this project's: column-major 3x3 matrices (element
// c[col][row], like the glm-style mat3 of lib/common.h:25-100), plain
// structs, no cooperative-groups dependency.
#pragma once

#include <math_constants.h>

#include <cstdint>
#include <cuda_runtime.h>

namespace splat {

struct M3 {
    float c[3][3];  // c[col][row]
};

__device__ __forceinline__ M3 m3(float a00, float a10, float a20, float a01, float a11,
                                 float a21, float a02, float a12, float a22) {
    // (col 0 rows 0..2, col 1 rows 0..2, col 2 rows 0..2)
    M3 m;
    m.c[0][0] = a00; m.c[0][1] = a10; m.c[0][2] = a20;
    m.c[1][0] = a01; m.c[1][1] = a11; m.c[1][2] = a21;
    m.c[2][0] = a02; m.c[2][1] = a12; m.c[2][2] = a22;
    return m;
}

__device__ __forceinline__ M3 m3_diag(float d) { return m3(d, 0.f, 0.f, 0.f, d, 0.f, 0.f, 0.f, d); }

// (a*b)[row r][col c] = sum_k a[row r][k] * b[k][col c], k = 0,1,2 left to right.
__device__ __forceinline__ M3 mul(const M3 &a, const M3 &b) {
    M3 o;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            o.c[c][r] = a.c[0][r] * b.c[c][0] + a.c[1][r] * b.c[c][1] + a.c[2][r] * b.c[c][2];
    return o;
}

__device__ __forceinline__ M3 add(const M3 &a, const M3 &b) {
    M3 o;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) o.c[c][r] = a.c[c][r] + b.c[c][r];
    return o;
}

__device__ __forceinline__ M3 tr(const M3 &a) {
    M3 o;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) o.c[c][r] = a.c[r][c];
    return o;
}

// Rotation from a (w, x, y, z) quaternion (helpers.h:140-153).
__device__ __forceinline__ M3 quat_rot(float4 q) {
    const float w = q.x, x = q.y, y = q.z, z = q.w;
    return m3(1.f - 2.f * (y * y + z * z), 2.f * (x * y + w * z), 2.f * (x * z - w * y),
              2.f * (x * y - w * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z + w * x),
              2.f * (x * z + w * y), 2.f * (y * z - w * x), 1.f - 2.f * (x * x + y * y));
}

__device__ __forceinline__ M3 scale_mat(float3 s, float glob) {
    M3 S = m3_diag(1.f);
    S.c[0][0] = glob * s.x;
    S.c[1][1] = glob * s.y;
    S.c[2][2] = glob * s.z;
    return S;
}

// Upper triangle of R S S^T R^T (forward.cu:547-568).
__device__ __forceinline__ void cov3d_from(float3 s, float glob, float4 q, float cov[6]) {
    const M3 R = quat_rot(q);
    const M3 S = scale_mat(s, glob);
    const M3 M = mul(R, S);
    const M3 C = mul(M, tr(M));
    cov[0] = C.c[0][0];
    cov[1] = C.c[0][1];
    cov[2] = C.c[0][2];
    cov[3] = C.c[1][1];
    cov[4] = C.c[1][2];
    cov[5] = C.c[2][2];
}

// Rotation block of a row-major 4x4 view matrix as a column-major M3.
__device__ __forceinline__ M3 view_rot(const float *v) {
    return m3(v[0], v[4], v[8], v[1], v[5], v[9], v[2], v[6], v[10]);
}

// R p + t for the row-major view matrix (helpers.h:101-108).
__device__ __forceinline__ float3 view_xform(const float *v, float3 p) {
    return make_float3(v[0] * p.x + v[1] * p.y + v[2] * p.z + v[3],
                       v[4] * p.x + v[5] * p.y + v[6] * p.z + v[7],
                       v[8] * p.x + v[9] * p.y + v[10] * p.z + v[11]);
}

// R^T p (helpers.h:90-98).
__device__ __forceinline__ float3 view_rot_T(const float *v, float3 p) {
    return make_float3(v[0] * p.x + v[4] * p.y + v[8] * p.z, v[1] * p.x + v[5] * p.y + v[9] * p.z,
                       v[2] * p.x + v[6] * p.y + v[10] * p.z);
}

// Camera-space mean through W (forward.cu:491-495, backward.cu:446-450).
__device__ __forceinline__ float3 cam_point(const M3 &W, const float *v, float3 m) {
    return make_float3(W.c[0][0] * m.x + W.c[1][0] * m.y + W.c[2][0] * m.z + v[3],
                       W.c[0][1] * m.x + W.c[1][1] * m.y + W.c[2][1] * m.z + v[7],
                       W.c[0][2] * m.x + W.c[1][2] * m.y + W.c[2][2] * m.z + v[11]);
}

// EWA splat of the 3D covariance (forward.cu:465-544): 2D covariance with the
// 0.3 px low-pass added, and the density compensation factor.
__device__ __forceinline__ void ewa_cov2d(float3 mean, const float cov3d[6], const float *v,
                                          float fx, float fy, float tanx, float tany,
                                          float3 &cov2d, float &comp) {
    const M3 W = view_rot(v);
    float3 t = cam_point(W, v, mean);
    const float limx = 1.3f * tanx;
    const float limy = 1.3f * tany;
    t.x = t.z * fminf(limx, fmaxf(-limx, t.x / t.z));
    t.y = t.z * fminf(limy, fmaxf(-limy, t.y / t.z));
    const float rz = 1.f / t.z;
    const float rz2 = rz * rz;
    const M3 J = m3(fx * rz, 0.f, 0.f, 0.f, fy * rz, 0.f, -fx * t.x * rz2, -fy * t.y * rz2, 0.f);
    const M3 T = mul(J, W);
    const M3 V = m3(cov3d[0], cov3d[1], cov3d[2], cov3d[1], cov3d[3], cov3d[4], cov3d[2],
                    cov3d[4], cov3d[5]);
    const M3 C = mul(mul(T, V), tr(T));
    const float c00 = C.c[0][0], c11 = C.c[1][1], c01 = C.c[0][1];
    const float det_orig = c00 * c11 - c01 * c01;
    cov2d.x = c00 + 0.3f;
    cov2d.y = c01;
    cov2d.z = c11 + 0.3f;
    const float det_blur = cov2d.x * cov2d.z - cov2d.y * cov2d.y;
    comp = sqrtf(fmaxf(0.f, det_orig / det_blur));
}

// Conic (inverse 2D covariance) and the 3-sigma radius (helpers.h:34-57).
__device__ __forceinline__ bool conic_radius(float3 cov2d, float3 &conic, float &radius) {
    const float det = cov2d.x * cov2d.z - cov2d.y * cov2d.y;
    if (det == 0.f) return false;
    const float inv_det = 1.f / det;
    conic.x = cov2d.z * inv_det;
    conic.y = -cov2d.y * inv_det;
    conic.z = cov2d.x * inv_det;
    const float b = 0.5f * (cov2d.x + cov2d.z);
    const float v1 = b + sqrtf(fmaxf(0.1f, b * b - det));
    const float v2 = b - sqrtf(fmaxf(0.1f, b * b - det));
    radius = ceilf(3.f * sqrtf(fmaxf(v1, v2)));
    return true;
}

// Pixel-space projection of a camera-space point (helpers.h:122-128).
__device__ __forceinline__ float2 to_pixel(float fx, float fy, float cx, float cy, float3 p) {
    const float rw = 1.f / (p.z + 1e-6f);
    const float2 q = make_float2(p.x * rw, p.y * rw);
    return make_float2(q.x * fx + cx, q.y * fy + cy);
}

// Tile-space bounding box, inclusive min / exclusive max, clamped to the
// tile grid (helpers.h:9-32).  The float->int conversions are the
// saturating round-toward-zero conversions of the device.
struct TileRect {
    unsigned x0, y0, x1, y1;
};

__device__ __forceinline__ unsigned clamp_tile(int v, unsigned hi) {
    const unsigned u = (unsigned)max(0, v);
    return u < hi ? u : hi;
}

__device__ __forceinline__ TileRect tile_rect(float2 center, float radius, unsigned tiles_x,
                                              unsigned tiles_y, unsigned bw) {
    const float cx = center.x / (float)bw;
    const float cy = center.y / (float)bw;
    const float rx = radius / (float)bw;
    const float ry = radius / (float)bw;
    TileRect r;
    r.x0 = clamp_tile((int)(cx - rx), tiles_x);
    r.x1 = clamp_tile((int)(cx + rx + 1), tiles_x);
    r.y0 = clamp_tile((int)(cy - ry), tiles_y);
    r.y1 = clamp_tile((int)(cy + ry + 1), tiles_y);
    return r;
}

// Gaussian falloff exponent at a pixel offset (forward.cu:424-426):
// 0.5 * (a dx dx + c dy dy) + b dx dy, written with the explicit roundings
// that the reference's expression compiles to -- the inner sum fuses its left
// product, the outer sum fuses b dx dy onto the scaled inner sum.  (Measured:
// this form reproduces the reference's image bit for bit at 1920x1080, the
// other fusion orders do not.)  Spelling the roundings out keeps the result
// independent of how the compiler would otherwise share products between
// pixels that have the same dx or dy.
__device__ __forceinline__ float falloff(float a, float b, float c, float dx, float dy) {
    const float inner = __fmaf_rn(__fmul_rn(a, dx), dx, __fmul_rn(__fmul_rn(c, dy), dy));
    return __fmaf_rn(__fmul_rn(b, dx), dy, __fmul_rn(0.5f, inner));
}

// pix_out + c * vis and acc + T * bg of forward.cu:443-459 (one fused
// multiply-add each).
__device__ __forceinline__ float blend(float acc, float c, float w) { return __fmaf_rn(c, w, acc); }

// ---------------------------------------------------------------------------
// Per-Gaussian rasterizer records.
//
//
// Record (3 x float4):  r0 = (x, y, conic a, conic b)
//                       r1 = (conic c, opacity, red, green)
//                       r2 = (blue, hx, hy, tag)
// (tag: 0 for a single view; for batched views the scene Gaussian's index,
// as int bits, that receives the colour and opacity gradients.)
// Outside the box |px - x| <= hx, |py - y| <= hy no pixel centre passes the
// test alpha >= 1/255 in the rasterizers' fp32 arithmetic.  hx = +inf means
// "no bound proven" (never culled); hx = -inf means "no pixel anywhere".
//
// Why the box is safe: for a positive-definite conic A the exact exponent is
// sigma = d^T A d / 2, and alpha >= 1/255 needs sigma <= thr = ln(255 o).
// The ellipse d^T A d <= q has half-extents sqrt(q (A^-1)_xx), sqrt(q (A^-1)_yy)
// with (A^-1)_xx = c / det, (A^-1)_yy = a / det.  The fp32 exponent differs
// from the exact one by at most 12 kappa 2^-24 of it, kappa = the condition
// number <= tr^2 / det; boxes are only built when tr^2 / det <= 1e4, so that
// is below 1% and q = 2 (thr + 0.01) / 0.98 covers it, the 0.01 absorbing the
// error of __expf and of the product o * exp.  det is formed with Kahan's
// error-free 2x2 determinant (within 2 ulp however much a c and b^2 cancel);
// logf and sqrtf are within 1 ulp; the half-extents get a further 0.1% and
// 0.01 px, and Gaussians centred more than 1e5 px away are never culled, so
// fp32 rounding of x +- hx cannot shrink the box.

constexpr float kCullMargin = 0.01f;
constexpr float kCullSigmaFactor = 0.98f;
constexpr float kCullMaxCond = 1e4f;
constexpr float kCullFarPx = 1e5f;

// The record of one Gaussian (xy, conic, opacity, colour; tag as above).
__device__ __forceinline__ void write_record(float4 *r, float2 xy, float3 conic, float o,
                                             float3 rgb, float tag) {
    const float ca = conic.x, cb = conic.y, cc = conic.z;
    float hx = CUDART_INF_F, hy = CUDART_INF_F;
    // det = a c - b^2 (Kahan): w = b*b rounded, e = its rounding error
    const float w = cb * cb;
    const float e = fmaf(cb, cb, -w);
    const float det = fmaf(ca, cc, -w) - e;
    const float trc = ca + cc;
    const bool finite = isfinite(xy.x) && isfinite(xy.y) && fabsf(xy.x) < kCullFarPx &&
                        fabsf(xy.y) < kCullFarPx && isfinite(o) && isfinite(ca) &&
                        isfinite(cb) && isfinite(cc) && isfinite(det);
    if (finite && ca > 0.f && cc > 0.f && det > 0.f && trc * trc <= kCullMaxCond * det && o > 0.f) {
        const float q = 2.f * (logf(255.f * o) + kCullMargin) / kCullSigmaFactor;
        if (q <= 0.f) {
            hx = hy = -CUDART_INF_F;
        } else {
            const float ex = sqrtf(q * cc / det) * 1.001f + 0.01f;
            const float ey = sqrtf(q * ca / det) * 1.001f + 0.01f;
            if (ex < kCullFarPx && ey < kCullFarPx) {
                hx = ex;
                hy = ey;
            }
        }
    }
    r[0] = make_float4(xy.x, xy.y, ca, cb);
    r[1] = make_float4(cc, o, rgb.x, rgb.y);
    r[2] = make_float4(rgb.z, hx, hy, tag);
}

}  // namespace splat
