// project.cu -- projection forward (fused with the tile-count scan) and
// projection backward.
//
// Forward: one thread per Gaussian, 4096 Gaussians per 512-thread block.
// Blocks take their partition from a ticket counter so that partitions start
// in order; each block scans its tile counts in registers/shared memory and
// resolves its exclusive prefix with a warp-parallel decoupled look-back,
// then writes cum_tiles_hit directly: one launch replaces the reference's
// projection kernel + CUB scan + eight memsets + three host synchronisations
// (lib/ops.cu:12-61).
#include <algorithm>

#include "project_math.cuh"
#include "splat_internal.cuh"

namespace splat {

// A block of 512 threads projects a partition of up to 4096 Gaussians, up
// to eight rounds of 512 consecutive ones: few partitions keep the look-back
// chain short (its inclusive prefixes advance by one window of partitions per
// L2 round trip), and two blocks fit on an SM.  Small inputs take fewer
// rounds per block so that every SM still gets work.
constexpr int kProjThreads = 512;
constexpr int kProjRounds = 8;  // at most
constexpr int kProjWarps = kProjThreads / 32;

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
    int rounds;  // rounds of kProjThreads Gaussians per partition, 1..kProjRounds
    // optional (rec non-null): the rasterizers' record of each Gaussian
    // (write_record) from its projection and its colour and opacity, which
    // makes the separate packing pass unnecessary
    const float *colors, *opac;
    float4 *rec;
};

// Inclusive scan over the block of one value per thread; returns the
// thread's inclusive sum and leaves the block total in *total.
__device__ __forceinline__ unsigned long long block_scan(unsigned long long v,
                                                         unsigned long long *s_warp,
                                                         unsigned long long *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kProjWarps ? s_warp[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        if (lane < kProjWarps) s_warp[lane] = w;
    }
    __syncthreads();
    const unsigned long long r = v + (warp ? s_warp[warp - 1] : 0ull);
    *total = s_warp[kProjWarps - 1];
    __syncthreads();  // s_warp is reused by the next round
    return r;
}

// Projects Gaussian i and writes every output of it (forward.cu:37-116; the
// reference's memsets provide the zeros of culled Gaussians); returns its
// tile count.
__device__ __forceinline__ uint32_t project_store(const ProjFwdArgs &a, const ProjCam &cam, int i) {
    const ProjOut o = project_one(cam, a.means3d + 3 * (size_t)i, a.scales + 3 * (size_t)i,
                                  a.quats + 4 * (size_t)i);
#pragma unroll
    for (int k = 0; k < 6; ++k) a.cov3d[6 * (size_t)i + k] = o.cov[k];
    a.xys[2 * (size_t)i] = o.center.x;
    a.xys[2 * (size_t)i + 1] = o.center.y;
    a.depths[i] = o.depth;
    a.radii[i] = o.radius;
    a.conics[3 * (size_t)i] = o.conic.x;
    a.conics[3 * (size_t)i + 1] = o.conic.y;
    a.conics[3 * (size_t)i + 2] = o.conic.z;
    a.comp[i] = o.comp;
    a.ntiles[i] = (int32_t)o.hits;
    if (a.rec)
        write_record(a.rec + 3 * (size_t)i, o.center, o.conic, a.opac[i],
                     make_float3(a.colors[3 * (size_t)i], a.colors[3 * (size_t)i + 1],
                                 a.colors[3 * (size_t)i + 2]),
                     0.f);
    return o.hits;
}

// Without cum_tiles_hit only the intersection total is wanted: one Gaussian
// per thread, no scan and no partition order, the block's tile counts summed
// (warp reductions, then one 64-bit atomic per block).
constexpr int kProjTotalThreads = 256;

__global__ void __launch_bounds__(kProjTotalThreads) project_fwd_total_kernel(ProjFwdArgs a) {
    __shared__ unsigned s_warp[kProjTotalThreads / 32];
    const ProjCam cam{a.viewmat, a.glob_scale, a.fx, a.fy, a.cx, a.cy, a.tanx, a.tany,
                      a.clip, a.tiles_x, a.tiles_y, a.bw};
    const int i = blockIdx.x * kProjTotalThreads + threadIdx.x;
    const uint32_t hits = i < a.n ? project_store(a, cam, i) : 0u;
    const unsigned w = __reduce_add_sync(0xffffffffu, hits);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long sum = 0;
#pragma unroll
        for (int k = 0; k < kProjTotalThreads / 32; ++k) sum += s_warp[k];
        if (sum) {
            const unsigned long long old =
                atomicAdd(reinterpret_cast<unsigned long long *>(a.total), sum);
            if (old + sum > 0x7fffffffull) raise_status(a.status, DEV_SCAN_OVERFLOW);
        }
    }
}

__global__ void __launch_bounds__(kProjThreads) project_fwd_kernel(ProjFwdArgs a) {
    __shared__ int s_part;
    __shared__ unsigned long long s_warp[kProjWarps];
    __shared__ unsigned long long s_prefix;
    if (threadIdx.x == 0) s_part = (int)atomicAdd(&a.words[0], 1ull);
    __syncthreads();
    const int part = s_part;
    const ProjCam cam{a.viewmat, a.glob_scale, a.fx, a.fy, a.cx, a.cy, a.tanx, a.tany,
                      a.clip, a.tiles_x, a.tiles_y, a.bw};

    // forward.cu:37-116, every output written (the reference's memsets
    // provide the zeros of culled Gaussians); inclusive scan per round
    const int part_size = a.rounds * kProjThreads;
    unsigned long long incl[kProjRounds];
    unsigned long long run = 0;
#pragma unroll
    for (int r = 0; r < kProjRounds; ++r) {
        if (r >= a.rounds) break;
        const int i = part * part_size + r * kProjThreads + threadIdx.x;
        const uint32_t hits = i < a.n ? project_store(a, cam, i) : 0u;
        unsigned long long round_total;
        incl[r] = run + block_scan(hits, s_warp, &round_total);
        run += round_total;
    }
    // partition prefix by decoupled look-back (64-bit carries)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        unsigned long long *words = a.words + 1;
        unsigned long long excl = 0;
        if (part == 0) {
            if (lane == 0) publish(&words[0], kFlagPrefix | (run & kValueMask));
        } else {
            if (lane == 0) publish(&words[part], kFlagAggregate | (run & kValueMask));
            excl = warp_lookback(words, part, a.spin_limit, a.status);
            if (lane == 0) publish(&words[part], kFlagPrefix | ((excl + run) & kValueMask));
        }
        if (lane == 0) {
            s_prefix = excl;
            const int nparts = (a.n + part_size - 1) / part_size;
            if (part == nparts - 1) {
                const unsigned long long total = excl + run;
                *a.total = (int64_t)total;
                if (total > 0x7fffffffull) raise_status(a.status, DEV_SCAN_OVERFLOW);
            }
        }
    }
    __syncthreads();
    const unsigned long long prefix = s_prefix;
#pragma unroll
    for (int r = 0; r < kProjRounds; ++r) {
        if (r >= a.rounds) break;
        const int i = part * part_size + r * kProjThreads + threadIdx.x;
        // int32 wrap, as the reference's int32 scan
        if (i < a.n) a.cum[i] = (int32_t)(uint32_t)(prefix + incl[r]);
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

// One Gaussian per thread; v_cov2d and v_cov3d only when asked for.
__global__ void __launch_bounds__(256) project_bwd_kernel(ProjBwdArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    ProjVjp g;
    if (a.radii[i] > 0) {
        const ProjCam cam{a.viewmat, a.glob_scale, a.fx, a.fy, 0.f, 0.f, 0.f, 0.f, 0.f, 0u, 0u, 0u};
        g = project_vjp_one(cam, a.means3d + 3 * (size_t)i, a.scales + 3 * (size_t)i,
                            a.quats + 4 * (size_t)i, a.cov3d + 6 * (size_t)i,
                            a.conics + 3 * (size_t)i, a.comp[i], a.v_xy + 2 * (size_t)i,
                            a.v_depth[i], a.v_conic + 3 * (size_t)i, a.v_comp[i]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a.v_mean3d[3 * i + k] = g.vmean[k];
        a.v_scale[3 * i + k] = g.vscale[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) a.v_quat[4 * i + k] = g.vquat[k];
    if (a.v_cov2d) {
#pragma unroll
        for (int k = 0; k < 3; ++k) a.v_cov2d[3 * i + k] = g.vc2[k];
    }
    if (a.v_cov3d) {
#pragma unroll
        for (int k = 0; k < 6; ++k) a.v_cov3d[6 * i + k] = g.vc3[k];
    }
}

// ---------------------------------------------------------------------------
// Host launchers.

// colors / opac / rec non-null: the packed records are written too.
int launch_project_fwd(const splat_params &p, const float *means3d, const float *scales,
                       const float *quats, const float *viewmat, float *cov3d, float *xys,
                       float *depths, int32_t *radii, float *conics, float *comp,
                       int32_t *ntiles, int32_t *cum, int64_t *total,
                       unsigned long long *words, const float *colors, const float *opac,
                       float *rec, cudaStream_t s) {
    const int n = (int)p.num_points;
    // rounds per partition: as few as keep the partitions within one wave of
    // two blocks per SM, at most 8
    const int rounds = std::max(1, std::min(kProjRounds, (n + 2 * 152 * kProjThreads - 1) /
                                                             (2 * 152 * kProjThreads)));
    const int nparts = (n + rounds * kProjThreads - 1) / (rounds * kProjThreads);
    if (cudaMemsetAsync(words, 0, sizeof(unsigned long long) * (size_t)(nparts + 1), s) != cudaSuccess)
        return check_launch("project_fwd workspace memset");
    // without cum_tiles_hit the blocks add their counts to the total
    if (!cum && cudaMemsetAsync(total, 0, sizeof(int64_t), s) != cudaSuccess)
        return check_launch("project_fwd total memset");
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
    a.rounds = rounds;
    a.colors = colors; a.opac = opac; a.rec = reinterpret_cast<float4 *>(rec);
    if (!cum) {
        project_fwd_total_kernel<<<(n + kProjTotalThreads - 1) / kProjTotalThreads,
                                   kProjTotalThreads, 0, s>>>(a);
        return check_launch("project_fwd_total_kernel");
    }
    project_fwd_kernel<<<nparts, kProjThreads, 0, s>>>(a);
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
