/*
 * splat_oracle.c -- CPU restatement of the jaxsplat render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke()
 * entry point and bench.py's cpu_baseline leg may call it, nothing in the
 * jaxsplat_gb300 product path does.
 *
 * It restates, step by step, what the reference's CUDA kernels compute:
 *   lib/kernels/forward.cu   project_gaussians_fwd (13-131),
 *                            map_gaussian_to_intersects (135-179),
 *                            get_tile_bin_edges (184-208),
 *                            rasterize_fwd (339-462),
 *                            project_cov3d_ewa (465-544),
 *                            scale_rot_to_cov3d (547-568)
 *   lib/kernels/backward.cu  rasterize_bwd (153-343),
 *                            project_gaussians_bwd (345-418),
 *                            project_cov3d_ewa_vjp (421-524),
 *                            scale_rot_to_cov3d_vjp (528-570)
 *   lib/kernels/helpers.h    bbox / conic / VJP / transform helpers (9-211)
 *   lib/common.h             column-major mat3 / mat2 semantics (25-137)
 *   lib/ops.cu               zero-initialised outputs (260-322, 356-394,
 *                            436-488, 534-602), the int32 inclusive scan
 *                            (607-643), the stable key sort over bits
 *                            [0, 32+msb) (723-757), the empty-list path
 *                            (119-127)
 *
 * Two builds come from this one source:
 *   ORACLE_F64 undefined: fp32 arithmetic.  Products that nvcc contracts
 *     into fused multiply-adds under its default -fmad=true are written as
 *     explicit fmaf() calls (FMA2/SOP/... below), and the file is compiled
 *     with -ffp-contract=off so that gcc adds no fusion of its own.  Division
 *     and square root are IEEE-rounded on both sides.  __expf has no exact
 *     CPU counterpart, so the rasterizer uses libm expf; pixels whose
 *     decisions sit on the alpha / transmittance thresholds may differ.
 *   ORACLE_F64 defined: the same algorithm evaluated in double (the FP64
 *     transcription used to state each output's error).
 *
 * All arrays are row-major and C-contiguous, with the reference's shapes.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_F64
typedef double real;
#define FMA(a, b, c) ((a) * (b) + (c))
#define RSQRT_(x) sqrt(x)
#define EXP_(x) exp(x)
#define CEIL_(x) ceil(x)
#define FMAX_(a, b) fmax((a), (b))
#define FMIN_(a, b) fmin((a), (b))
#define K(x) ((real)(x))
#define SYM(name) oracle64_##name
#else
typedef float real;
#define FMA(a, b, c) fmaf((a), (b), (c))
#define RSQRT_(x) sqrtf(x)
#define EXP_(x) expf(x)
#define CEIL_(x) ceilf(x)
#define FMAX_(a, b) fmaxf((a), (b))
#define FMIN_(a, b) fminf((a), (b))
#define K(x) ((real)(x##f))
#define SYM(name) oracle32_##name
#endif

#define API __attribute__((visibility("default")))

/* a*b + c*d as nvcc contracts it: the left product is fused. */
static inline real SOP(real a, real b, real c, real d) { return FMA(a, b, c * d); }
/* a*b - c*d: fma(a, b, -(c*d)). */
static inline real SOPM(real a, real b, real c, real d) { return FMA(a, b, -(c * d)); }
/* a0*b0 + a1*b1 + a2*b2 evaluated left to right with contraction. */
static inline real DOT3(real a0, real b0, real a1, real b1, real a2, real b2) {
    return FMA(a2, b2, FMA(a0, b0, a1 * b1));
}

/* float -> int32 with the GPU's saturating, NaN -> 0 conversion
 * (cvt.rzi.s32.f32 semantics; C leaves the out-of-range case undefined). */
static inline int32_t f2i_sat(real x) {
    if (x != x) return 0;
    if (x >= (real)2147483648.0) return INT32_MAX;
    if (x <= (real)-2147483648.0) return INT32_MIN;
    return (int32_t)x;
}

/* ------------------------------------------------------------------ */
/* Column-major 3x3 matrix: m[col][row], as lib/common.h:25-100.       */
typedef struct { real m[3][3]; } mat3;

static inline mat3 mat3_cols(real m00, real m10, real m20, real m01, real m11,
                             real m21, real m02, real m12, real m22) {
    /* argument order follows common.h:41-52: (col0 rows 0..2, col1, col2) */
    mat3 r;
    r.m[0][0] = m00; r.m[0][1] = m10; r.m[0][2] = m20;
    r.m[1][0] = m01; r.m[1][1] = m11; r.m[1][2] = m21;
    r.m[2][0] = m02; r.m[2][1] = m12; r.m[2][2] = m22;
    return r;
}

static inline mat3 mat3_diag(real d) {
    return mat3_cols(d, 0, 0, 0, d, 0, 0, 0, d);
}

/* common.h:59-71: out[c][r] = sum_k a[k][r] * b[c][k], k = 0,1,2 in order */
static inline mat3 mat3_mul(const mat3 *a, const mat3 *b) {
    mat3 o;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            o.m[c][r] = DOT3(a->m[0][r], b->m[c][0], a->m[1][r], b->m[c][1],
                             a->m[2][r], b->m[c][2]);
    return o;
}

static inline mat3 mat3_add(const mat3 *a, const mat3 *b) {
    mat3 o;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) o.m[c][r] = a->m[c][r] + b->m[c][r];
    return o;
}

static inline mat3 mat3_T(const mat3 *a) {
    mat3 o;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) o.m[c][r] = a->m[r][c];
    return o;
}

/* Column-major 2x2, common.h:102-137. */
typedef struct { real m[2][2]; } mat2;

static inline mat2 mat2_cols(real m00, real m10, real m01, real m11) {
    mat2 r;
    r.m[0][0] = m00; r.m[0][1] = m10; r.m[1][0] = m01; r.m[1][1] = m11;
    return r;
}

static inline mat2 mat2_mul(const mat2 *a, const mat2 *b) {
    return mat2_cols(SOP(a->m[0][0], b->m[0][0], a->m[1][0], b->m[0][1]),
                     SOP(a->m[0][1], b->m[0][0], a->m[1][1], b->m[0][1]),
                     SOP(a->m[0][0], b->m[1][0], a->m[1][0], b->m[1][1]),
                     SOP(a->m[0][1], b->m[1][0], a->m[1][1], b->m[1][1]));
}

static inline mat2 mat2_neg(const mat2 *a) {
    return mat2_cols(-a->m[0][0], -a->m[0][1], -a->m[1][0], -a->m[1][1]);
}

/* ------------------------------------------------------------------ */
/* helpers.h:101-108: R*p + t for a row-major [R|t] view matrix.      */
static inline void transform_4x3(const real *v, const real p[3], real out[3]) {
    for (int r = 0; r < 3; ++r)
        out[r] = DOT3(v[4 * r + 0], p[0], v[4 * r + 1], p[1], v[4 * r + 2], p[2]) +
                 v[4 * r + 3];
}

/* helpers.h:90-98: R^T * p, ignoring the translation column. */
static inline void transform_4x3_rot_T(const real *v, const real p[3], real out[3]) {
    for (int c = 0; c < 3; ++c)
        out[c] = DOT3(v[c], p[0], v[4 + c], p[1], v[8 + c], p[2]);
}

/* helpers.h:140-153: wxyz quaternion to rotation, column-major. */
static mat3 quat_to_rotmat(const real q[4]) {
    real w = q[0], x = q[1], y = q[2], z = q[3];
    return mat3_cols(K(1.0) - K(2.0) * SOP(y, y, z, z), K(2.0) * SOP(x, y, w, z),
                     K(2.0) * SOPM(x, z, w, y), K(2.0) * SOPM(x, y, w, z),
                     K(1.0) - K(2.0) * SOP(x, x, z, z), K(2.0) * SOP(y, z, w, x),
                     K(2.0) * SOP(x, z, w, y), K(2.0) * SOPM(y, z, w, x),
                     K(1.0) - K(2.0) * SOP(x, x, y, y));
}

/* helpers.h:194-201 */
static mat3 scale_to_mat(const real s[3], real glob) {
    mat3 S = mat3_diag(K(1.0));
    S.m[0][0] = glob * s[0];
    S.m[1][1] = glob * s[1];
    S.m[2][2] = glob * s[2];
    return S;
}

/* forward.cu:547-568 */
static void scale_rot_to_cov3d(const real s[3], real glob, const real q[4], real cov[6]) {
    mat3 R = quat_to_rotmat(q);
    mat3 S = scale_to_mat(s, glob);
    mat3 M = mat3_mul(&R, &S);
    mat3 Mt = mat3_T(&M);
    mat3 tmp = mat3_mul(&M, &Mt);
    cov[0] = tmp.m[0][0];
    cov[1] = tmp.m[0][1];
    cov[2] = tmp.m[0][2];
    cov[3] = tmp.m[1][1];
    cov[4] = tmp.m[1][2];
    cov[5] = tmp.m[2][2];
}

static mat3 view_rot(const real *v) {
    /* forward.cu:479-489: W[c][r] = viewmat[4r + c] */
    return mat3_cols(v[0], v[4], v[8], v[1], v[5], v[9], v[2], v[6], v[10]);
}

static void view_point(const mat3 *W, const real *v, const real mean[3], real t[3]) {
    /* forward.cu:491-495 */
    for (int r = 0; r < 3; ++r)
        t[r] = DOT3(W->m[0][r], mean[0], W->m[1][r], mean[1], W->m[2][r], mean[2]) +
               v[4 * r + 3];
}

/* forward.cu:465-544 */
static void project_cov3d_ewa(const real mean[3], const real cov3d[6], const real *v,
                              real fx, real fy, real tanx, real tany, real cov2d[3],
                              real *comp) {
    mat3 W = view_rot(v);
    real t[3];
    view_point(&W, v, mean, t);
    real limx = K(1.3) * tanx, limy = K(1.3) * tany;
    t[0] = t[2] * FMIN_(limx, FMAX_(-limx, t[0] / t[2]));
    t[1] = t[2] * FMIN_(limy, FMAX_(-limy, t[1] / t[2]));
    real rz = K(1.0) / t[2];
    real rz2 = rz * rz;
    mat3 J = mat3_cols(fx * rz, 0, 0, 0, fy * rz, 0, -fx * t[0] * rz2, -fy * t[1] * rz2, 0);
    mat3 T = mat3_mul(&J, &W);
    mat3 V = mat3_cols(cov3d[0], cov3d[1], cov3d[2], cov3d[1], cov3d[3], cov3d[4],
                       cov3d[2], cov3d[4], cov3d[5]);
    mat3 TV = mat3_mul(&T, &V);
    mat3 Tt = mat3_T(&T);
    mat3 cov = mat3_mul(&TV, &Tt);
    real c00 = cov.m[0][0], c11 = cov.m[1][1], c01 = cov.m[0][1];
    real det_orig = SOPM(c00, c11, c01, c01);
    cov2d[0] = c00 + K(0.3);
    cov2d[1] = c01;
    cov2d[2] = c11 + K(0.3);
    real det_blur = SOPM(cov2d[0], cov2d[2], cov2d[1], cov2d[1]);
    *comp = RSQRT_(FMAX_(K(0.0), det_orig / det_blur));
}

/* helpers.h:34-57 */
static int compute_cov2d_bounds(const real cov2d[3], real conic[3], real *radius) {
    real det = SOPM(cov2d[0], cov2d[2], cov2d[1], cov2d[1]);
    if (det == K(0.0)) return 0;
    real inv_det = K(1.0) / det;
    conic[0] = cov2d[2] * inv_det;
    conic[1] = -cov2d[1] * inv_det;
    conic[2] = cov2d[0] * inv_det;
    real b = K(0.5) * (cov2d[0] + cov2d[2]);
    real disc = FMA(b, b, -det);
    real v1 = b + RSQRT_(FMAX_(K(0.1), disc));
    real v2 = b - RSQRT_(FMAX_(K(0.1), disc));
    *radius = CEIL_(K(3.0) * RSQRT_(FMAX_(v1, v2)));
    return 1;
}

/* helpers.h:9-32: tile-space bbox, inclusive min / exclusive max, clamped. */
static void tile_bbox(real cx, real cy, real radius, unsigned tiles_x, unsigned tiles_y,
                      unsigned bw, unsigned out[4]) {
    real bwf = (real)bw;
    real tcx = cx / bwf, tcy = cy / bwf;
    real tr = radius / bwf;
    int32_t a;
    a = f2i_sat(tcx - tr); a = a > 0 ? a : 0;
    out[0] = (unsigned)a < tiles_x ? (unsigned)a : tiles_x;
    a = f2i_sat(tcx + tr + K(1.0)); a = a > 0 ? a : 0;
    out[2] = (unsigned)a < tiles_x ? (unsigned)a : tiles_x;
    a = f2i_sat(tcy - tr); a = a > 0 ? a : 0;
    out[1] = (unsigned)a < tiles_y ? (unsigned)a : tiles_y;
    a = f2i_sat(tcy + tr + K(1.0)); a = a > 0 ? a : 0;
    out[3] = (unsigned)a < tiles_y ? (unsigned)a : tiles_y;
}

static inline float as_f32(real x) { return (float)x; }

/* ------------------------------------------------------------------ */
/* Projection forward, forward.cu:13-131 plus ops.cu:52-57 (scan).     */
API void SYM(project_fwd)(int n, const real *means3d, const real *scales, real glob_scale,
                          const real *quats, const real *viewmat, real fx, real fy,
                          real cx, real cy, unsigned img_w, unsigned img_h,
                          unsigned block_width, real clip_thresh, real *cov3d, real *xys,
                          real *depths, int32_t *radii, real *conics, real *compensation,
                          int32_t *num_tiles_hit, int32_t *cum_tiles_hit) {
    unsigned tiles_x = (img_w + block_width - 1) / block_width;
    unsigned tiles_y = (img_h + block_width - 1) / block_width;
    /* forward.cu:70-71: evaluated in double, then rounded to the kernel's float */
    real tanx = (real)(0.5 * (double)img_w / (double)fx);
    real tany = (real)(0.5 * (double)img_h / (double)fy);
    /* ops.cu:260-322: every output starts at zero */
    memset(cov3d, 0, sizeof(real) * 6 * (size_t)n);
    memset(xys, 0, sizeof(real) * 2 * (size_t)n);
    memset(depths, 0, sizeof(real) * (size_t)n);
    memset(radii, 0, sizeof(int32_t) * (size_t)n);
    memset(conics, 0, sizeof(real) * 3 * (size_t)n);
    memset(compensation, 0, sizeof(real) * (size_t)n);
    memset(num_tiles_hit, 0, sizeof(int32_t) * (size_t)n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const real *p = means3d + 3 * (size_t)i;
        real pv[3];
        transform_4x3(viewmat, p, pv);
        if (pv[2] <= clip_thresh) continue; /* helpers.h:204-211 */
        real *c3 = cov3d + 6 * (size_t)i;
        scale_rot_to_cov3d(scales + 3 * (size_t)i, glob_scale, quats + 4 * (size_t)i, c3);
        real cov2d[3], comp;
        project_cov3d_ewa(p, c3, viewmat, fx, fy, tanx, tany, cov2d, &comp);
        real conic[3], radius;
        if (!compute_cov2d_bounds(cov2d, conic, &radius)) continue;
        conics[3 * (size_t)i + 0] = conic[0];
        conics[3 * (size_t)i + 1] = conic[1];
        conics[3 * (size_t)i + 2] = conic[2];
        /* helpers.h:122-128 */
        real rw = K(1.0) / (pv[2] + K(1e-6));
        real px = FMA(pv[0] * rw, fx, cx);
        real py = FMA(pv[1] * rw, fy, cy);
        unsigned bb[4];
        tile_bbox(px, py, radius, tiles_x, tiles_y, block_width, bb);
        int32_t area = (int32_t)((bb[2] - bb[0]) * (bb[3] - bb[1]));
        if (area <= 0) continue;
        num_tiles_hit[i] = area;
        depths[i] = pv[2];
        radii[i] = f2i_sat(radius);
        xys[2 * (size_t)i + 0] = px;
        xys[2 * (size_t)i + 1] = py;
        compensation[i] = comp;
    }
    /* ops.cu:607-643: inclusive int32 scan (wraps like the device scan) */
    uint32_t acc = 0;
    for (int i = 0; i < n; ++i) {
        acc += (uint32_t)num_tiles_hit[i];
        cum_tiles_hit[i] = (int32_t)acc;
    }
}

/* forward.cu:135-179: one (key, id) pair per touched tile, row-major tile
 * order, written at offset cum_tiles_hit[i-1]. */
API void SYM(map_intersects)(int n, const real *xys, const real *depths, const int32_t *radii,
                             const int32_t *cum_tiles_hit, unsigned img_w, unsigned img_h,
                             unsigned block_width, int64_t *isect_ids, int32_t *gaussian_ids) {
    unsigned tiles_x = (img_w + block_width - 1) / block_width;
    unsigned tiles_y = (img_h + block_width - 1) / block_width;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int i = 0; i < n; ++i) {
        if (radii[i] <= 0) continue;
        unsigned bb[4];
        tile_bbox(xys[2 * (size_t)i], xys[2 * (size_t)i + 1], (real)radii[i], tiles_x,
                  tiles_y, block_width, bb);
        int32_t cur = i == 0 ? 0 : cum_tiles_hit[i - 1];
        float d = as_f32(depths[i]);
        int32_t dbits;
        memcpy(&dbits, &d, 4);
        int64_t depth_id = (int64_t)dbits; /* sign-extended, forward.cu:168 */
        for (unsigned y = bb[1]; y < bb[3]; ++y)
            for (unsigned x = bb[0]; x < bb[2]; ++x) {
                int64_t tile = (int64_t)(uint32_t)(y * tiles_x + x);
                isect_ids[cur] = (int64_t)((uint64_t)tile << 32) | depth_id;
                gaussian_ids[cur] = i;
                ++cur;
            }
    }
}

/* ops.cu:723-724: bits sorted = 32 + msb, msb = bit length of n_tiles + 1 */
API int SYM(sort_end_bit)(unsigned n_tiles) {
    int msb = 0;
    while ((n_tiles >> msb) != 0) ++msb;
    return 32 + msb + 1;
}

/* ops.cu:728-757: stable ascending sort on the low end_bit bits of the key,
 * values permuted alongside (what an LSD radix sort computes).  Stable
 * bottom-up merge sort on the masked key. */
API void SYM(sort_pairs)(int64_t count, const int64_t *keys_in, const int32_t *vals_in,
                         int end_bit, int64_t *keys_out, int32_t *vals_out) {
    if (count <= 0) return;
    uint64_t mask = end_bit >= 64 ? ~0ull : ((1ull << end_bit) - 1ull);
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)count);
    int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (size_t)count);
    uint64_t *mk = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        idx[i] = i;
        mk[i] = (uint64_t)keys_in[i] & mask;
    }
    for (int64_t width = 1; width < count; width *= 2) {
#pragma omp parallel for schedule(static)
        for (int64_t lo = 0; lo < count; lo += 2 * width) {
            int64_t mid = lo + width < count ? lo + width : count;
            int64_t hi = lo + 2 * width < count ? lo + 2 * width : count;
            int64_t a = lo, b = mid, o = lo;
            while (a < mid && b < hi) tmp[o++] = (mk[idx[b]] < mk[idx[a]]) ? idx[b++] : idx[a++];
            while (a < mid) tmp[o++] = idx[a++];
            while (b < hi) tmp[o++] = idx[b++];
        }
        int64_t *sw = idx; idx = tmp; tmp = sw;
    }
    for (int64_t i = 0; i < count; ++i) {
        keys_out[i] = keys_in[idx[i]];
        vals_out[i] = vals_in[idx[i]];
    }
    free(idx); free(tmp); free(mk);
}

/* forward.cu:184-208 plus ops.cu:482-488 (tiles with no entry stay (0,0)). */
API void SYM(tile_bin_edges)(int64_t count, const int64_t *sorted_keys, int n_tiles,
                             int32_t *tile_bins) {
    memset(tile_bins, 0, sizeof(int32_t) * 2 * (size_t)n_tiles);
    for (int64_t i = 0; i < count; ++i) {
        int32_t cur = (int32_t)(sorted_keys[i] >> 32);
        if (i == 0) tile_bins[2 * cur] = 0;
        if (i == count - 1) tile_bins[2 * cur + 1] = (int32_t)count;
        if (i == 0) continue;
        int32_t prev = (int32_t)(sorted_keys[i - 1] >> 32);
        if (prev != cur) {
            tile_bins[2 * prev + 1] = (int32_t)i;
            tile_bins[2 * cur] = (int32_t)i;
        }
    }
}

/* Per-pixel Gaussian falloff exponent, forward.cu:424-426 with nvcc's
 * contraction: the inner sum fuses its left product, the outer sum fuses
 * b dx dy onto the 0.5-scaled inner sum (the form that reproduces the
 * reference kernel's image bit for bit). */
static inline real falloff(const real *conic, real dx, real dy) {
    real inner = FMA(conic[0] * dx, dx, conic[2] * dy * dy);
    return FMA(conic[1] * dx, dy, K(0.5) * inner);
}

/* forward.cu:339-462 (and ops.cu:119-127 when there is no intersection). */
API void SYM(rasterize_fwd)(unsigned img_w, unsigned img_h, unsigned block_width,
                            int64_t num_intersects, const int32_t *ids_sorted,
                            const int32_t *tile_bins, const real *xys, const real *conics,
                            const real *colors, const real *opacities, const real *background,
                            real *final_Ts, int32_t *final_idx, real *out_img) {
    size_t npix = (size_t)img_w * img_h;
    memset(final_Ts, 0, sizeof(real) * npix);
    memset(final_idx, 0, sizeof(int32_t) * npix);
    if (num_intersects == 0) {
        for (size_t p = 0; p < npix; ++p)
            for (int c = 0; c < 3; ++c) out_img[3 * p + c] = background[c];
        return;
    }
    unsigned tiles_x = (img_w + block_width - 1) / block_width;
    unsigned tiles_y = (img_h + block_width - 1) / block_width;
    const real thresh = K(1.0) / K(255.0);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (unsigned ty = 0; ty < tiles_y; ++ty)
        for (unsigned tx = 0; tx < tiles_x; ++tx) {
            int tile = (int)(ty * tiles_x + tx);
            int32_t lo = tile_bins[2 * tile], hi = tile_bins[2 * tile + 1];
            for (unsigned py = ty * block_width; py < (ty + 1) * block_width && py < img_h; ++py)
                for (unsigned px = tx * block_width; px < (tx + 1) * block_width && px < img_w;
                     ++px) {
                    real fx = (real)px + K(0.5), fy = (real)py + K(0.5);
                    real T = K(1.0);
                    int32_t cur = 0;
                    real acc[3] = {0, 0, 0};
                    for (int32_t k = lo; k < hi; ++k) {
                        int32_t g = ids_sorted[k];
                        const real *con = conics + 3 * (size_t)g;
                        real dx = xys[2 * (size_t)g] - fx, dy = xys[2 * (size_t)g + 1] - fy;
                        real sigma = falloff(con, dx, dy);
                        real alpha = FMIN_(K(0.999), opacities[g] * EXP_(-sigma));
                        if (sigma < K(0.0) || alpha < thresh) continue;
                        real nextT = T * (K(1.0) - alpha);
                        if (nextT <= K(1e-4)) break;
                        real vis = alpha * T;
                        for (int c = 0; c < 3; ++c)
                            acc[c] = FMA(colors[3 * (size_t)g + c], vis, acc[c]);
                        T = nextT;
                        cur = k;
                    }
                    size_t pid = (size_t)py * img_w + px;
                    final_Ts[pid] = T;
                    final_idx[pid] = cur;
                    for (int c = 0; c < 3; ++c) out_img[3 * pid + c] = FMA(T, background[c], acc[c]);
                }
        }
}

static inline void atomic_add_real(real *p, real v) {
#pragma omp atomic
    *p += v;
}

/* backward.cu:153-343: reverse traversal from final_idx, transmittance
 * recovered by division, alpha clamp 0.99.  Sums are accumulated per pixel
 * in a fixed order (tile-parallel when OpenMP is on). */
API void SYM(rasterize_bwd)(unsigned img_w, unsigned img_h, unsigned block_width, int n,
                            int64_t num_intersects, const int32_t *ids_sorted,
                            const int32_t *tile_bins, const real *xys, const real *conics,
                            const real *colors, const real *opacities, const real *background,
                            const real *final_Ts, const int32_t *final_idx, const real *v_out,
                            const real *v_out_alpha, real *v_xy, real *v_xy_abs, real *v_conic,
                            real *v_colors, real *v_opacity) {
    memset(v_xy, 0, sizeof(real) * 2 * (size_t)n);
    memset(v_xy_abs, 0, sizeof(real) * 2 * (size_t)n);
    memset(v_conic, 0, sizeof(real) * 3 * (size_t)n);
    memset(v_colors, 0, sizeof(real) * 3 * (size_t)n);
    memset(v_opacity, 0, sizeof(real) * (size_t)n);
    if (num_intersects == 0) return; /* ops.cu:184-186 */
    unsigned tiles_x = (img_w + block_width - 1) / block_width;
    unsigned tiles_y = (img_h + block_width - 1) / block_width;
    const real thresh = K(1.0) / K(255.0);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (unsigned ty = 0; ty < tiles_y; ++ty)
        for (unsigned tx = 0; tx < tiles_x; ++tx) {
            int tile = (int)(ty * tiles_x + tx);
            int32_t lo = tile_bins[2 * tile];
            for (unsigned py = ty * block_width; py < (ty + 1) * block_width && py < img_h; ++py)
                for (unsigned px = tx * block_width; px < (tx + 1) * block_width && px < img_w;
                     ++px) {
                    size_t pid = (size_t)py * img_w + px;
                    real fx = (real)px + K(0.5), fy = (real)py + K(0.5);
                    real T_final = final_Ts[pid];
                    real T = T_final;
                    real buf[3] = {0, 0, 0};
                    const real *vo = v_out + 3 * pid;
                    real voa = v_out_alpha[pid];
                    for (int32_t k = final_idx[pid]; k >= lo; --k) {
                        int32_t g = ids_sorted[k];
                        const real *con = conics + 3 * (size_t)g;
                        real dx = xys[2 * (size_t)g] - fx, dy = xys[2 * (size_t)g + 1] - fy;
                        real sigma = falloff(con, dx, dy);
                        real vis = EXP_(-sigma);
                        real opac = opacities[g];
                        real alpha = FMIN_(K(0.99), opac * vis);
                        if (sigma < K(0.0) || alpha < thresh) continue;
                        real ra = K(1.0) / (K(1.0) - alpha);
                        T *= ra;
                        real fac = alpha * T;
                        const real *rgb = colors + 3 * (size_t)g;
                        real v_alpha = 0;
                        for (int c = 0; c < 3; ++c) v_alpha += (rgb[c] * T - buf[c] * ra) * vo[c];
                        v_alpha += T_final * ra * voa;
                        for (int c = 0; c < 3; ++c) v_alpha += -T_final * ra * background[c] * vo[c];
                        for (int c = 0; c < 3; ++c) buf[c] += rgb[c] * fac;
                        real v_sigma = -opac * vis * v_alpha;
                        real vcx = K(0.5) * v_sigma * dx * dx;
                        real vcy = v_sigma * dx * dy;
                        real vcz = K(0.5) * v_sigma * dy * dy;
                        real vx = v_sigma * (con[0] * dx + con[1] * dy);
                        real vy = v_sigma * (con[1] * dx + con[2] * dy);
                        for (int c = 0; c < 3; ++c) atomic_add_real(&v_colors[3 * (size_t)g + c], fac * vo[c]);
                        atomic_add_real(&v_conic[3 * (size_t)g + 0], vcx);
                        atomic_add_real(&v_conic[3 * (size_t)g + 1], vcy);
                        atomic_add_real(&v_conic[3 * (size_t)g + 2], vcz);
                        atomic_add_real(&v_xy[2 * (size_t)g + 0], vx);
                        atomic_add_real(&v_xy[2 * (size_t)g + 1], vy);
                        atomic_add_real(&v_xy_abs[2 * (size_t)g + 0], vx < 0 ? -vx : vx);
                        atomic_add_real(&v_xy_abs[2 * (size_t)g + 1], vy < 0 ? -vy : vy);
                        atomic_add_real(&v_opacity[g], vis * v_alpha);
                    }
                }
        }
}

/* helpers.h:60-71 */
static void cov2d_to_conic_vjp(const real conic[3], const real vconic[3], real vcov[3]) {
    mat2 X = mat2_cols(conic[0], conic[1], conic[1], conic[2]);
    mat2 G = mat2_cols(vconic[0], vconic[1] / K(2.0), vconic[1] / K(2.0), vconic[2]);
    mat2 nX = mat2_neg(&X);
    mat2 a = mat2_mul(&nX, &G);
    mat2 s = mat2_mul(&a, &X);
    vcov[0] = s.m[0][0];
    vcov[1] = s.m[1][0] + s.m[0][1];
    vcov[2] = s.m[1][1];
}

/* helpers.h:73-87 (double-precision literals in the reference, so the
 * arithmetic is carried in double before rounding back). */
static void cov2d_to_compensation_vjp(real comp, const real conic[3], real vcomp, real vcov[3]) {
    real inv_det = SOPM(conic[0], conic[2], conic[1], conic[1]);
    real omsc = K(1.0) - comp * comp;
    real vsc = (real)((double)vcomp * 0.5 / ((double)comp + 1e-6));
    vcov[0] = (real)((double)vcov[0] + (double)vsc * ((double)(omsc * conic[0]) - 0.3 * (double)inv_det));
    vcov[1] = (real)((double)vcov[1] + 2.0 * (double)vsc * (double)(omsc * conic[1]));
    vcov[2] = (real)((double)vcov[2] + (double)vsc * ((double)(omsc * conic[2]) - 0.3 * (double)inv_det));
}

/* backward.cu:421-524 (no frustum clamp in the adjoint). */
static void project_cov3d_ewa_vjp(const real mean[3], const real cov3d[6], const real *v,
                                  real fx, real fy, const real vcov2d[3], real vmean[3],
                                  real vcov3d[6]) {
    mat3 W = view_rot(v);
    real t[3];
    view_point(&W, v, mean, t);
    real rz = K(1.0) / t[2];
    real rz2 = rz * rz;
    mat3 J = mat3_cols(fx * rz, 0, 0, 0, fy * rz, 0, -fx * t[0] * rz2, -fy * t[1] * rz2, 0);
    mat3 V = mat3_cols(cov3d[0], cov3d[1], cov3d[2], cov3d[1], cov3d[3], cov3d[4], cov3d[2],
                       cov3d[4], cov3d[5]);
    mat3 vc = mat3_cols(vcov2d[0], K(0.5) * vcov2d[1], 0, K(0.5) * vcov2d[1], vcov2d[2], 0, 0,
                        0, 0);
    mat3 T = mat3_mul(&J, &W);
    mat3 Tt = mat3_T(&T);
    mat3 Vt = mat3_T(&V);
    mat3 a = mat3_mul(&Tt, &vc);
    mat3 vV = mat3_mul(&a, &T);
    mat3 b1 = mat3_mul(&vc, &T);
    mat3 b2 = mat3_mul(&b1, &Vt);
    mat3 vcT = mat3_T(&vc);
    mat3 c1 = mat3_mul(&vcT, &T);
    mat3 c2 = mat3_mul(&c1, &V);
    mat3 vT = mat3_add(&b2, &c2);
    vcov3d[0] = vV.m[0][0];
    vcov3d[1] = vV.m[0][1] + vV.m[1][0];
    vcov3d[2] = vV.m[0][2] + vV.m[2][0];
    vcov3d[3] = vV.m[1][1];
    vcov3d[4] = vV.m[1][2] + vV.m[2][1];
    vcov3d[5] = vV.m[2][2];
    mat3 Wt = mat3_T(&W);
    mat3 vJ = mat3_mul(&vT, &Wt);
    real rz3 = rz2 * rz;
    real vt0 = -fx * rz2 * vJ.m[2][0];
    real vt1 = -fy * rz2 * vJ.m[2][1];
    real vt2 = -fx * rz2 * vJ.m[0][0] + K(2.0) * fx * t[0] * rz3 * vJ.m[2][0] -
               fy * rz2 * vJ.m[1][1] + K(2.0) * fy * t[1] * rz3 * vJ.m[2][1];
    vmean[0] += vt0 * W.m[0][0] + vt1 * W.m[0][1] + vt2 * W.m[0][2];
    vmean[1] += vt0 * W.m[1][0] + vt1 * W.m[1][1] + vt2 * W.m[1][2];
    vmean[2] += vt0 * W.m[2][0] + vt1 * W.m[2][1] + vt2 * W.m[2][2];
}

/* helpers.h:155-192 */
static void quat_to_rotmat_vjp(const real q[4], const mat3 *vR, real vq[4]) {
    real w = q[0], x = q[1], y = q[2], z = q[3];
    const real(*R)[3] = vR->m;
    vq[0] = K(2.0) * (x * (R[1][2] - R[2][1]) + y * (R[2][0] - R[0][2]) + z * (R[0][1] - R[1][0]));
    vq[1] = K(2.0) * (-K(2.0) * x * (R[1][1] + R[2][2]) + y * (R[0][1] + R[1][0]) +
                      z * (R[0][2] + R[2][0]) + w * (R[1][2] - R[2][1]));
    vq[2] = K(2.0) * (x * (R[0][1] + R[1][0]) - K(2.0) * y * (R[0][0] + R[2][2]) +
                      z * (R[1][2] + R[2][1]) + w * (R[2][0] - R[0][2]));
    vq[3] = K(2.0) * (x * (R[0][2] + R[2][0]) + y * (R[1][2] + R[2][1]) -
                      K(2.0) * z * (R[0][0] + R[1][1]) + w * (R[0][1] - R[1][0]));
}

/* backward.cu:528-570 */
static void scale_rot_to_cov3d_vjp(const real s[3], real glob, const real q[4],
                                   const real vc[6], real vs[3], real vq[4]) {
    mat3 vV = mat3_cols(vc[0], K(0.5) * vc[1], K(0.5) * vc[2], K(0.5) * vc[1], vc[3],
                        K(0.5) * vc[4], K(0.5) * vc[2], K(0.5) * vc[4], vc[5]);
    mat3 R = quat_to_rotmat(q);
    mat3 S = scale_to_mat(s, glob);
    mat3 M = mat3_mul(&R, &S);
    mat3 two = mat3_diag(K(2.0)); /* `v_V * M * 2.f` converts 2.f to 2*I */
    mat3 vVM = mat3_mul(&vV, &M);
    mat3 vM = mat3_mul(&vVM, &two);
    for (int k = 0; k < 3; ++k)
        vs[k] = (R.m[k][0] * vM.m[k][0] + R.m[k][1] * vM.m[k][1] + R.m[k][2] * vM.m[k][2]) * glob;
    mat3 vR = mat3_mul(&vM, &S);
    quat_to_rotmat_vjp(q, &vR, vq);
}

/* backward.cu:345-418 plus ops.cu:356-394 (zeroed outputs). */
API void SYM(project_bwd)(int n, const real *means3d, const real *scales, real glob_scale,
                          const real *quats, const real *viewmat, real fx, real fy,
                          const real *cov3d, const int32_t *radii, const real *conics,
                          const real *compensation, const real *v_xy, const real *v_depth,
                          const real *v_conic, const real *v_compensation, real *v_cov2d,
                          real *v_cov3d, real *v_mean3d, real *v_scale, real *v_quat) {
    memset(v_cov2d, 0, sizeof(real) * 3 * (size_t)n);
    memset(v_cov3d, 0, sizeof(real) * 6 * (size_t)n);
    memset(v_mean3d, 0, sizeof(real) * 3 * (size_t)n);
    memset(v_scale, 0, sizeof(real) * 3 * (size_t)n);
    memset(v_quat, 0, sizeof(real) * 4 * (size_t)n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (radii[i] <= 0) continue;
        const real *p = means3d + 3 * (size_t)i;
        real pv[3];
        transform_4x3(viewmat, p, pv);
        /* helpers.h:131-138 */
        real rw = K(1.0) / (pv[2] + K(1e-6));
        real vpx = fx * v_xy[2 * (size_t)i], vpy = fy * v_xy[2 * (size_t)i + 1];
        real vview[3] = {vpx * rw, vpy * rw, -(vpx * pv[0] + vpy * pv[1]) * rw * rw};
        real *vm = v_mean3d + 3 * (size_t)i;
        transform_4x3_rot_T(viewmat, vview, vm);
        real vz = v_depth[i];
        vm[0] += viewmat[8] * vz;
        vm[1] += viewmat[9] * vz;
        vm[2] += viewmat[10] * vz;
        real *vc2 = v_cov2d + 3 * (size_t)i;
        cov2d_to_conic_vjp(conics + 3 * (size_t)i, v_conic + 3 * (size_t)i, vc2);
        cov2d_to_compensation_vjp(compensation[i], conics + 3 * (size_t)i, v_compensation[i], vc2);
        project_cov3d_ewa_vjp(p, cov3d + 6 * (size_t)i, viewmat, fx, fy, vc2, vm,
                              v_cov3d + 6 * (size_t)i);
        scale_rot_to_cov3d_vjp(scales + 3 * (size_t)i, glob_scale, quats + 4 * (size_t)i,
                               v_cov3d + 6 * (size_t)i, v_scale + 3 * (size_t)i,
                               v_quat + 4 * (size_t)i);
    }
}

API void SYM(set_threads)(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

API int SYM(max_threads)(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
