// project_math.cuh -- projection of one Gaussian and its vector-Jacobian
// product, shared by the single-view kernels (project.cu) and the batched
// multi-view kernels (batch.cu) so that both compute the same bits.
#pragma once

#include "splat_math.cuh"

namespace splat {

// Camera and tile grid of one view.
struct ProjCam {
    const float *viewmat;  // row-major 4x4, world -> camera
    float glob_scale, fx, fy, cx, cy;
    float tanx, tany;  // 0.5 W / fx, 0.5 H / fy (forward.cu:70-71, evaluated in double)
    float clip;
    unsigned tiles_x, tiles_y, bw;
};

struct ProjOut {
    float cov[6];
    float3 conic;
    float2 center;
    float depth, comp;
    int radius;
    uint32_t hits;
};

// forward.cu:37-116 for one Gaussian.  Every field is set; the zeros are the
// values the reference's memsets leave for culled Gaussians (ops.cu:260-322):
// cov3d is kept for every Gaussian in front of the near plane, the conic
// whenever det != 0, the rest only when the tile area is positive.
__device__ __forceinline__ ProjOut project_one(const ProjCam &cam, const float *mean,
                                               const float *scale, const float *quat) {
    ProjOut o;
#pragma unroll
    for (int k = 0; k < 6; ++k) o.cov[k] = 0.f;
    o.conic = make_float3(0.f, 0.f, 0.f);
    o.center = make_float2(0.f, 0.f);
    o.depth = 0.f;
    o.comp = 0.f;
    o.radius = 0;
    o.hits = 0;
    const float3 pw = make_float3(mean[0], mean[1], mean[2]);
    const float3 pv = view_xform(cam.viewmat, pw);
    if (!(pv.z <= cam.clip)) {
        const float3 s = make_float3(scale[0], scale[1], scale[2]);
        const float4 q = make_float4(quat[0], quat[1], quat[2], quat[3]);
        cov3d_from(s, cam.glob_scale, q, o.cov);
        float3 cov2d;
        float comp;
        ewa_cov2d(pw, o.cov, cam.viewmat, cam.fx, cam.fy, cam.tanx, cam.tany, cov2d, comp);
        float radius;
        if (conic_radius(cov2d, o.conic, radius)) {
            const float2 c = to_pixel(cam.fx, cam.fy, cam.cx, cam.cy, pv);
            const TileRect r = tile_rect(c, radius, cam.tiles_x, cam.tiles_y, cam.bw);
            const int32_t area = (int32_t)((r.x1 - r.x0) * (r.y1 - r.y0));
            if (area > 0) {
                o.hits = (uint32_t)area;
                o.depth = pv.z;
                o.radius = (int)radius;
                o.center = c;
                o.comp = comp;
            }
        }
    }
    return o;
}

__device__ __forceinline__ M3 m3_scaled_sym(const float v[6]) {
    // symmetric matrix from upper-triangle cotangents, off-diagonals halved
    return m3(v[0], 0.5f * v[1], 0.5f * v[2], 0.5f * v[1], v[3], 0.5f * v[4], 0.5f * v[2],
              0.5f * v[4], v[5]);
}

struct ProjVjp {
    float vmean[3] = {0.f, 0.f, 0.f}, vscale[3] = {0.f, 0.f, 0.f};
    float vquat[4] = {0.f, 0.f, 0.f, 0.f}, vc2[3] = {0.f, 0.f, 0.f};
    float vc3[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
};

// backward.cu:345-418 for one Gaussian with radius > 0, with the VJP helpers
// helpers.h:60-192 and backward.cu:421-570 (no frustum clamp in the adjoint,
// double-precision literals in the compensation VJP).  Uses cam.viewmat,
// glob_scale, fx and fy.
__device__ __forceinline__ ProjVjp project_vjp_one(const ProjCam &cam, const float *mean,
                                                   const float *scale, const float *quat,
                                                   const float *c3, const float *conic,
                                                   float comp_in, const float *v_xy,
                                                   float v_depth, const float *v_conic,
                                                   float v_comp) {
    ProjVjp r;
    float *vmean = r.vmean, *vscale = r.vscale, *vquat = r.vquat, *vc2 = r.vc2, *vc3 = r.vc3;
    const float *v = cam.viewmat;
    const float fx = cam.fx, fy = cam.fy;
    const float3 pw = make_float3(mean[0], mean[1], mean[2]);
    const float3 pv = view_xform(v, pw);
    // helpers.h:131-138 then the transposed rotation
    const float2 vxy = make_float2(v_xy[0], v_xy[1]);
    {
        const float rw = 1.f / (pv.z + 1e-6f);
        const float2 vp = make_float2(fx * vxy.x, fy * vxy.y);
        const float3 vv = make_float3(vp.x * rw, vp.y * rw, -(vp.x * pv.x + vp.y * pv.y) * rw * rw);
        const float3 m = view_rot_T(v, vv);
        vmean[0] = m.x;
        vmean[1] = m.y;
        vmean[2] = m.z;
    }
    const float vz = v_depth;
    vmean[0] += v[8] * vz;
    vmean[1] += v[9] * vz;
    vmean[2] += v[10] * vz;

    // conic -> cov2d (helpers.h:60-71)
    const float3 con = make_float3(conic[0], conic[1], conic[2]);
    const float3 vcon = make_float3(v_conic[0], v_conic[1], v_conic[2]);
    {
        // -X G X with X = [[a,b],[b,c]], G = [[va, vb/2],[vb/2, vc]] (column-major 2x2)
        const float x00 = -con.x, x10 = -con.y, x01 = -con.y, x11 = -con.z;
        const float g00 = vcon.x, g10 = vcon.y / 2.f, g01 = vcon.y / 2.f, g11 = vcon.z;
        const float p00 = x00 * g00 + x01 * g10, p10 = x10 * g00 + x11 * g10;
        const float p01 = x00 * g01 + x01 * g11, p11 = x10 * g01 + x11 * g11;
        const float s00 = p00 * con.x + p01 * con.y, s10 = p10 * con.x + p11 * con.y;
        const float s01 = p00 * con.y + p01 * con.z, s11 = p10 * con.y + p11 * con.z;
        vc2[0] = s00;
        vc2[1] = s01 + s10;
        vc2[2] = s11;
    }
    // compensation -> cov2d (helpers.h:73-87, double-precision literals).
    // With a zero cotangent (render's case) every term is a zero product, so
    // the block -- double arithmetic, slow on this GPU -- is skipped.
    if (v_comp != 0.f) {
        const float comp = comp_in;
        const float inv_det = con.x * con.z - con.y * con.y;
        const float omsc = 1 - comp * comp;
        const float vsc = v_comp * 0.5 / (comp + 1e-6);
        vc2[0] += vsc * (omsc * con.x - 0.3 * inv_det);
        vc2[1] += 2 * vsc * (omsc * con.y);
        vc2[2] += vsc * (omsc * con.z - 0.3 * inv_det);
    }
    // cov2d -> cov3d and mean (backward.cu:421-524, no frustum clamp)
    const M3 W = view_rot(v);
    const float3 t = cam_point(W, v, pw);
    const float rz = 1.f / t.z;
    const float rz2 = rz * rz;
    const M3 J = m3(fx * rz, 0.f, 0.f, 0.f, fy * rz, 0.f, -fx * t.x * rz2, -fy * t.y * rz2, 0.f);
    const M3 V = m3(c3[0], c3[1], c3[2], c3[1], c3[3], c3[4], c3[2], c3[4], c3[5]);
    const M3 G = m3(vc2[0], 0.5f * vc2[1], 0.f, 0.5f * vc2[1], vc2[2], 0.f, 0.f, 0.f, 0.f);
    const M3 T = mul(J, W);
    const M3 Tt = tr(T);
    const M3 vV = mul(mul(Tt, G), T);
    const M3 vT = add(mul(mul(G, T), tr(V)), mul(mul(tr(G), T), V));
    vc3[0] = vV.c[0][0];
    vc3[1] = vV.c[0][1] + vV.c[1][0];
    vc3[2] = vV.c[0][2] + vV.c[2][0];
    vc3[3] = vV.c[1][1];
    vc3[4] = vV.c[1][2] + vV.c[2][1];
    vc3[5] = vV.c[2][2];
    const M3 vJ = mul(vT, tr(W));
    const float rz3 = rz2 * rz;
    const float vt0 = -fx * rz2 * vJ.c[2][0];
    const float vt1 = -fy * rz2 * vJ.c[2][1];
    const float vt2 = -fx * rz2 * vJ.c[0][0] + 2.f * fx * t.x * rz3 * vJ.c[2][0] -
                      fy * rz2 * vJ.c[1][1] + 2.f * fy * t.y * rz3 * vJ.c[2][1];
    vmean[0] += vt0 * W.c[0][0] + vt1 * W.c[0][1] + vt2 * W.c[0][2];
    vmean[1] += vt0 * W.c[1][0] + vt1 * W.c[1][1] + vt2 * W.c[1][2];
    vmean[2] += vt0 * W.c[2][0] + vt1 * W.c[2][1] + vt2 * W.c[2][2];

    // cov3d -> scale, quaternion (backward.cu:528-570, helpers.h:155-192)
    const float3 s = make_float3(scale[0], scale[1], scale[2]);
    const float4 q = make_float4(quat[0], quat[1], quat[2], quat[3]);
    const M3 vVs = m3_scaled_sym(vc3);
    const M3 R = quat_rot(q);
    const M3 S = scale_mat(s, cam.glob_scale);
    const M3 M = mul(R, S);
    const M3 vM = mul(mul(vVs, M), m3_diag(2.f));
#pragma unroll
    for (int k = 0; k < 3; ++k)
        vscale[k] = (R.c[k][0] * vM.c[k][0] + R.c[k][1] * vM.c[k][1] + R.c[k][2] * vM.c[k][2]) *
                    cam.glob_scale;
    const M3 vR = mul(vM, S);
    const float w = q.x, x = q.y, y = q.z, z = q.w;
    const auto &g = vR.c;
    vquat[0] = 2.f * (x * (g[1][2] - g[2][1]) + y * (g[2][0] - g[0][2]) + z * (g[0][1] - g[1][0]));
    vquat[1] = 2.f * (-2.f * x * (g[1][1] + g[2][2]) + y * (g[0][1] + g[1][0]) +
                      z * (g[0][2] + g[2][0]) + w * (g[1][2] - g[2][1]));
    vquat[2] = 2.f * (x * (g[0][1] + g[1][0]) - 2.f * y * (g[0][0] + g[2][2]) +
                      z * (g[1][2] + g[2][1]) + w * (g[2][0] - g[0][2]));
    vquat[3] = 2.f * (x * (g[0][2] + g[2][0]) + y * (g[1][2] + g[2][1]) -
                      2.f * z * (g[0][0] + g[1][1]) + w * (g[0][1] - g[1][0]));
    return r;
}

}  // namespace splat
