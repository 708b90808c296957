// project.cu -- projection forward (fused with the tile-count scan) and
// projection backward.
//
// Forward: one thread per Gaussian, 256 Gaussians per block.  Blocks take
// their partition from a ticket counter so that partitions start in order;
// each block scans its tile counts in registers/shared memory and resolves
// its exclusive prefix with a warp-parallel decoupled look-back, then writes
// cum_tiles_hit directly: one launch replaces the reference's projection
// kernel + CUB scan + eight memsets + three host synchronisations
// (lib/ops.cu:12-61).
#include "splat_internal.cuh"
#include "splat_math.cuh"

namespace splat {

constexpr int kProjBlock = 256;

struct ProjFwdArgs {
    int n;
    const float *means3d, *scales, *quats, *viewmat;
    float glob_scale, fx, fy, cx, cy, tanx, tany, clip;
    unsigned tiles_x, tiles_y, bw;
    float *cov3d, *xys, *depths, *conics, *comp;
    int32_t *radii, *ntiles, *cum;
    int64_t *total;
    unsigned long long *words;  // [0] ticket counter, [1 + b] look-back word of partition b
    uint32_t *status;
    uint32_t spin_limit;
};

__global__ void __launch_bounds__(kProjBlock) project_fwd_kernel(ProjFwdArgs a) {
    __shared__ int s_part;
    __shared__ unsigned long long s_warp[kProjBlock / 32];
    __shared__ unsigned long long s_prefix;
    if (threadIdx.x == 0) s_part = (int)atomicAdd(&a.words[0], 1ull);
    __syncthreads();
    const int part = s_part;
    const int i = part * kProjBlock + threadIdx.x;

    uint32_t hits = 0;
    if (i < a.n) {
        // forward.cu:37-116, every output written (the reference's memsets
        // provide the zeros of culled Gaussians).
        float cov[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float3 conic = make_float3(0.f, 0.f, 0.f);
        float2 center = make_float2(0.f, 0.f);
        float depth = 0.f, comp_out = 0.f;
        int radius_out = 0;
        const float3 pw = make_float3(a.means3d[3 * i], a.means3d[3 * i + 1], a.means3d[3 * i + 2]);
        const float3 pv = view_xform(a.viewmat, pw);
        if (!(pv.z <= a.clip)) {
            const float3 s = make_float3(a.scales[3 * i], a.scales[3 * i + 1], a.scales[3 * i + 2]);
            const float4 q = make_float4(a.quats[4 * i], a.quats[4 * i + 1], a.quats[4 * i + 2],
                                         a.quats[4 * i + 3]);
            cov3d_from(s, a.glob_scale, q, cov);
            float3 cov2d;
            float comp;
            ewa_cov2d(pw, cov, a.viewmat, a.fx, a.fy, a.tanx, a.tany, cov2d, comp);
            float radius;
            if (conic_radius(cov2d, conic, radius)) {
                const float2 c = to_pixel(a.fx, a.fy, a.cx, a.cy, pv);
                const TileRect r = tile_rect(c, radius, a.tiles_x, a.tiles_y, a.bw);
                const int32_t area = (int32_t)((r.x1 - r.x0) * (r.y1 - r.y0));
                if (area > 0) {
                    hits = (uint32_t)area;
                    depth = pv.z;
                    radius_out = (int)radius;
                    center = c;
                    comp_out = comp;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) a.cov3d[6 * i + k] = cov[k];
        a.xys[2 * i] = center.x;
        a.xys[2 * i + 1] = center.y;
        a.depths[i] = depth;
        a.radii[i] = radius_out;
        a.conics[3 * i] = conic.x;
        a.conics[3 * i + 1] = conic.y;
        a.conics[3 * i + 2] = conic.z;
        a.comp[i] = comp_out;
        a.ntiles[i] = (int32_t)hits;
    }

    // Block-wide inclusive scan of the tile counts (64-bit carries).
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long v = hits;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kProjBlock / 32 ? s_warp[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        if (lane < kProjBlock / 32) s_warp[lane] = w;  // inclusive over warps
        const unsigned long long block_total = __shfl_sync(0xffffffffu, w, kProjBlock / 32 - 1);
        unsigned long long *words = a.words + 1;
        unsigned long long excl = 0;
        if (part == 0) {
            if (lane == 0) publish(&words[0], kFlagPrefix | (block_total & kValueMask));
        } else {
            if (lane == 0) publish(&words[part], kFlagAggregate | (block_total & kValueMask));
            excl = warp_lookback(words, part, a.spin_limit, a.status);
            if (lane == 0) publish(&words[part], kFlagPrefix | ((excl + block_total) & kValueMask));
        }
        if (lane == 0) {
            s_prefix = excl;
            const int nparts = (a.n + kProjBlock - 1) / kProjBlock;
            if (part == nparts - 1) {
                const unsigned long long total = excl + block_total;
                *a.total = (int64_t)total;
                if (total > 0x7fffffffull) raise_status(a.status, DEV_SCAN_OVERFLOW);
            }
        }
    }
    __syncthreads();
    if (i < a.n) {
        const unsigned long long incl = s_prefix + (warp ? s_warp[warp - 1] : 0ull) + v;
        a.cum[i] = (int32_t)(uint32_t)incl;  // int32 wrap, as the reference's int32 scan
    }
}

// ---------------------------------------------------------------------------
// Projection backward (backward.cu:345-418 and the VJP helpers
// helpers.h:60-192, backward.cu:421-570).

struct ProjBwdArgs {
    int n;
    const float *means3d, *scales, *quats, *viewmat, *cov3d, *conics, *comp;
    const int32_t *radii;
    const float *v_xy, *v_depth, *v_conic, *v_comp;
    float glob_scale, fx, fy;
    float *v_mean3d, *v_scale, *v_quat, *v_cov2d, *v_cov3d;
};

__device__ __forceinline__ M3 m3_scaled_sym(const float v[6]) {
    // symmetric matrix from upper-triangle cotangents, off-diagonals halved
    return m3(v[0], 0.5f * v[1], 0.5f * v[2], 0.5f * v[1], v[3], 0.5f * v[4], 0.5f * v[2],
              0.5f * v[4], v[5]);
}

__global__ void __launch_bounds__(256) project_bwd_kernel(ProjBwdArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float vmean[3] = {0.f, 0.f, 0.f}, vscale[3] = {0.f, 0.f, 0.f};
    float vquat[4] = {0.f, 0.f, 0.f, 0.f}, vc2[3] = {0.f, 0.f, 0.f};
    float vc3[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (a.radii[i] > 0) {
        const float *v = a.viewmat;
        const float3 pw = make_float3(a.means3d[3 * i], a.means3d[3 * i + 1], a.means3d[3 * i + 2]);
        const float3 pv = view_xform(v, pw);
        // helpers.h:131-138 then the transposed rotation
        const float2 vxy = make_float2(a.v_xy[2 * i], a.v_xy[2 * i + 1]);
        {
            const float rw = 1.f / (pv.z + 1e-6f);
            const float2 vp = make_float2(a.fx * vxy.x, a.fy * vxy.y);
            const float3 vv = make_float3(vp.x * rw, vp.y * rw, -(vp.x * pv.x + vp.y * pv.y) * rw * rw);
            const float3 m = view_rot_T(v, vv);
            vmean[0] = m.x;
            vmean[1] = m.y;
            vmean[2] = m.z;
        }
        const float vz = a.v_depth[i];
        vmean[0] += v[8] * vz;
        vmean[1] += v[9] * vz;
        vmean[2] += v[10] * vz;

        // conic -> cov2d (helpers.h:60-71)
        const float3 con = make_float3(a.conics[3 * i], a.conics[3 * i + 1], a.conics[3 * i + 2]);
        const float3 vcon = make_float3(a.v_conic[3 * i], a.v_conic[3 * i + 1], a.v_conic[3 * i + 2]);
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
        // compensation -> cov2d (helpers.h:73-87, double-precision literals)
        {
            const float comp = a.comp[i];
            const float inv_det = con.x * con.z - con.y * con.y;
            const float omsc = 1 - comp * comp;
            const float vsc = a.v_comp[i] * 0.5 / (comp + 1e-6);
            vc2[0] += vsc * (omsc * con.x - 0.3 * inv_det);
            vc2[1] += 2 * vsc * (omsc * con.y);
            vc2[2] += vsc * (omsc * con.z - 0.3 * inv_det);
        }
        // cov2d -> cov3d and mean (backward.cu:421-524, no frustum clamp)
        const M3 W = view_rot(v);
        const float3 t = cam_point(W, v, pw);
        const float rz = 1.f / t.z;
        const float rz2 = rz * rz;
        const M3 J = m3(a.fx * rz, 0.f, 0.f, 0.f, a.fy * rz, 0.f, -a.fx * t.x * rz2,
                        -a.fy * t.y * rz2, 0.f);
        const float *c3 = a.cov3d + 6 * i;
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
        const float vt0 = -a.fx * rz2 * vJ.c[2][0];
        const float vt1 = -a.fy * rz2 * vJ.c[2][1];
        const float vt2 = -a.fx * rz2 * vJ.c[0][0] + 2.f * a.fx * t.x * rz3 * vJ.c[2][0] -
                          a.fy * rz2 * vJ.c[1][1] + 2.f * a.fy * t.y * rz3 * vJ.c[2][1];
        vmean[0] += vt0 * W.c[0][0] + vt1 * W.c[0][1] + vt2 * W.c[0][2];
        vmean[1] += vt0 * W.c[1][0] + vt1 * W.c[1][1] + vt2 * W.c[1][2];
        vmean[2] += vt0 * W.c[2][0] + vt1 * W.c[2][1] + vt2 * W.c[2][2];

        // cov3d -> scale, quaternion (backward.cu:528-570, helpers.h:155-192)
        const float3 s = make_float3(a.scales[3 * i], a.scales[3 * i + 1], a.scales[3 * i + 2]);
        const float4 q = make_float4(a.quats[4 * i], a.quats[4 * i + 1], a.quats[4 * i + 2],
                                     a.quats[4 * i + 3]);
        const M3 vVs = m3_scaled_sym(vc3);
        const M3 R = quat_rot(q);
        const M3 S = scale_mat(s, a.glob_scale);
        const M3 M = mul(R, S);
        const M3 vM = mul(mul(vVs, M), m3_diag(2.f));
#pragma unroll
        for (int k = 0; k < 3; ++k)
            vscale[k] = (R.c[k][0] * vM.c[k][0] + R.c[k][1] * vM.c[k][1] + R.c[k][2] * vM.c[k][2]) *
                        a.glob_scale;
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
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a.v_mean3d[3 * i + k] = vmean[k];
        a.v_scale[3 * i + k] = vscale[k];
        a.v_cov2d[3 * i + k] = vc2[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) a.v_quat[4 * i + k] = vquat[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) a.v_cov3d[6 * i + k] = vc3[k];
}

// ---------------------------------------------------------------------------
// Host launchers.

int launch_project_fwd(const splat_params &p, const float *means3d, const float *scales,
                       const float *quats, const float *viewmat, float *cov3d, float *xys,
                       float *depths, int32_t *radii, float *conics, float *comp,
                       int32_t *ntiles, int32_t *cum, int64_t *total,
                       unsigned long long *words, cudaStream_t s) {
    const int n = (int)p.num_points;
    const int nparts = (n + kProjBlock - 1) / kProjBlock;
    if (cudaMemsetAsync(words, 0, sizeof(unsigned long long) * (size_t)(nparts + 1), s) != cudaSuccess)
        return check_launch("project_fwd workspace memset");
    ProjFwdArgs a;
    a.n = n;
    a.means3d = means3d; a.scales = scales; a.quats = quats; a.viewmat = viewmat;
    a.glob_scale = p.glob_scale;
    a.fx = p.fx; a.fy = p.fy; a.cx = p.cx; a.cy = p.cy;
    // forward.cu:70-71: evaluated in double, rounded to float
    a.tanx = (float)(0.5 * (double)p.img_width / (double)p.fx);
    a.tany = (float)(0.5 * (double)p.img_height / (double)p.fy);
    a.clip = p.clip_thresh;
    a.tiles_x = tiles_x(p); a.tiles_y = tiles_y(p); a.bw = p.block_width;
    a.cov3d = cov3d; a.xys = xys; a.depths = depths; a.conics = conics; a.comp = comp;
    a.radii = radii; a.ntiles = ntiles; a.cum = cum; a.total = total;
    a.words = words;
    a.status = p.device_status;
    a.spin_limit = spin_limit(p);
    project_fwd_kernel<<<nparts, kProjBlock, 0, s>>>(a);
    return check_launch("project_fwd_kernel");
}

int launch_project_bwd(const splat_params &p, const float *means3d, const float *scales,
                       const float *quats, const float *viewmat, const float *cov3d,
                       const int32_t *radii, const float *conics, const float *comp,
                       const float *v_xy, const float *v_depth, const float *v_conic,
                       const float *v_comp, float *v_mean3d, float *v_scale, float *v_quat,
                       float *v_cov2d, float *v_cov3d, cudaStream_t s) {
    const int n = (int)p.num_points;
    ProjBwdArgs a;
    a.n = n;
    a.means3d = means3d; a.scales = scales; a.quats = quats; a.viewmat = viewmat;
    a.cov3d = cov3d; a.conics = conics; a.comp = comp; a.radii = radii;
    a.v_xy = v_xy; a.v_depth = v_depth; a.v_conic = v_conic; a.v_comp = v_comp;
    a.glob_scale = p.glob_scale; a.fx = p.fx; a.fy = p.fy;
    a.v_mean3d = v_mean3d; a.v_scale = v_scale; a.v_quat = v_quat;
    a.v_cov2d = v_cov2d; a.v_cov3d = v_cov3d;
    project_bwd_kernel<<<(n + 255) / 256, 256, 0, s>>>(a);
    return check_launch("project_bwd_kernel");
}

}  // namespace splat
