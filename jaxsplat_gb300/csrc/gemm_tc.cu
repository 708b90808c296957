// gemm_tc.cu -- BF16 GEMM with FP32 accumulation on the 5th-generation tensor
// cores (tcgen05), for the warm-start network's convolutions (as im2col
// GEMMs) and their gradients.
//
//   C[M,N] (fp32, row-major, ldc) (+)= op(A) x op(B)^T, bf16 operands:
//     A stored [M,K] (K-major) or [K,M] (MN-major: A^T row-major),
//     B stored [N,K] (K-major) or [K,N] (MN-major),
//   or, fused into the epilogue, y[M,N] = act(A B^T + bias) as bf16 (or fp32).
//
// One CTA of 128 threads computes a 128 x BN tile of C (BN = 32, 64 or 128,
// the smallest that covers N, so narrow layers waste no MMA columns; 64 or
// 128 when an operand is MN-major).  Operand tiles of 64 K-elements arrive by
// TMA (cp.async.bulk.tensor, tensor maps over this GPU's memory, no
// multicast) in the 128-byte-swizzled layouts the tensor cores read directly
// -- K-major: rows of 64 K-elements; MN-major: 64-element MN atoms of 64
// K-rows, so the weight-gradient products (reductions over the pixel rows of
// both operands) and the data-gradient product (the weights as stored) need
// no transposed copies -- through a ring of S stages: thread 0 (producer)
// waits for a stage's "empty" barrier and issues its tensor loads onto the
// stage's "full" barrier; thread 32 (MMA issuer) waits for "full", issues
// four tcgen05.mma (M 128, N BN, K 16) into a BN-column FP32 accumulator in
// tensor memory and commits them to the stage's "empty" barrier.  After the
// last stage a commit to "done" releases the epilogue: every warp reads its
// 32 accumulator lanes (= tile rows) with tcgen05.ld, adds the bias and
// applies the ReLU where asked, writes its 32-row slab into the (now idle)
// stage ring in the 128-byte-swizzled layout, and one lane stores the slab
// with a TMA tensor store -- or a TMA reduce-add for split-K partial sums and
// accumulation -- so C leaves in full 128-byte lines and the fp32 product of
// the fused forms is never stored and re-read.  (Outputs whose row stride or
// base is not 16-byte aligned, and 32-column bf16 tiles, are written from
// the registers instead.)
//
// Every wait is bounded: a barrier that does not flip within spin_limit
// polls sets DEV_LOOKBACK_TIMEOUT in the status word; the CTA then waits (again
// bounded) for its commits, skips the epilogue, frees its tensor memory and
// returns.
#include <cuda.h>  // CUtensorMap and its enums; the encoder comes from the driver entry point
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "splat_internal.cuh"

namespace splat {

constexpr int kGemmBM = 128;
constexpr int kGemmBK = 64;  // 64 bf16 = one 128-byte swizzle row
constexpr int kGemmThreads = 128;
constexpr int kGemmATile = kGemmBM * kGemmBK * 2;  // 16 KB

template <int BN>
constexpr int gemm_stage_bytes() {
    return kGemmATile + BN * kGemmBK * 2;
}
// Dynamic shared memory of a ring: S stages + alignment slack, and for
// MN-major operands 8 KB more past the ring, so that the tensor cores' reads
// through a 64-column MN-major descriptor stay inside this CTA's allocation
// whichever of its two strides (1024 and 8192 bytes) walks the K-row groups.
template <int BN, int S, bool kMN = false>
constexpr int gemm_smem() {
    return S * gemm_stage_bytes<BN>() + 1024 + (kMN ? 8192 : 0);
}

enum GemmOut { kOutF32 = 0, kOutBiasBF16 = 1, kOutBiasF32 = 2 };

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzled layout (rows of 128 bytes, 8-row / 1024-byte swizzle atoms, the
// stage buffers 1024-byte aligned): stride byte offset 1024 between 8-row
// groups, leading byte offset unused (encoded as 16), descriptor version 1,
// layout type 2 (128-byte swizzle).  The K-th 16-element slice of a row
// starts 32 K bytes into it: the hardware applies the swizzle to the
// address, so advancing the start address selects the slice.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Shared-memory matrix descriptor of an MN-major operand in the 128-byte
// swizzled layout: atoms of 64 MN-elements (one 128-byte row) x 8 K-rows
// (1024 bytes); stride byte offset 1024 between 8-K-row groups, leading byte
// offset 8192 between 64-element MN atoms (each tensor load brings one atom
// column of 64 K-rows), layout type 2.  The K-th 16-row slice starts
// 2048 K bytes in (two whole 8-row groups).
__device__ __forceinline__ uint64_t smem_desc_sw128_mn(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(8192u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f16: D fp32, A and B bf16; a_mn / b_mn
// mark an MN-major operand (bits 15 and 16).
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n, bool a_mn = false,
                                                 bool b_mn = false) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
           ((b_mn ? 1u : 0u) << 16) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Waits for the barrier's phase with mbarrier.try_wait, which suspends the
// thread until the phase completes or a time limit (the hint, ~1 us) passes;
// gives up after `limit` tries.  (Polling test_wait with a sleep between
// polls wakes up to one sleep late at every ring stage.)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity), "r"(1000u)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n"
                 ::"r"(bar), "r"(bytes)
                 : "memory");
}

// 2-D tensor load of the box at (x = K element, y = row) into shared memory,
// completing on `bar`.  x is a multiple of 64 elements (128 bytes).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// 2-D tensor store (or reduce-add into global) of the shared-memory box at
// `src` to (x = column, y = row); x a multiple of 32 fp32 / 64 bf16 (128
// bytes), both coordinates inside the tensor.  Completion through the
// thread's bulk async-group.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];\n" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(src), "r"(x), "r"(y)
                 : "memory");
}
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap *map, uint32_t src, int x,
                                                  int y) {
    asm volatile(
        "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.bulk_group [%0, {%2, %3}], [%1];\n" ::"l"(
            reinterpret_cast<uint64_t>(map)),
        "r"(src), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c,
                                             uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(addr), "r"(a), "r"(b), "r"(c),
                 "r"(d)
                 : "memory");
}

// Byte offset of a 16-byte chunk in a 1024-byte-aligned 128-byte-swizzled
// box: the chunk index (bits 4-6) XOR the 128-byte line index (bits 7-9).
__device__ __forceinline__ uint32_t swz128(uint32_t off) {
    return off ^ (((off >> 7) & 7u) << 4);
}

struct GemmArgs {
    float *C;               // kOutF32 / kOutBiasF32 output (ldc)
    __nv_bfloat16 *y16;     // kOutBiasBF16 output (ldc)
    const float *bias;      // [N], kOutBias*
    int M, N, K;
    int ldc;                // elements
    int accumulate;         // kOutF32: add to C instead of overwriting
    int relu;               // kOutBias*: max(., 0)
    int mode;               // GemmOut
    int ktiles_per;         // K tiles per CTA along grid z (split K: partial sums added atomically)
    int tma_out;            // the epilogue stores through map_c (TMA) instead of from registers
    uint32_t *status;
    uint32_t spin_limit;
};

// Epilogue of one row segment of 16 accumulator columns starting at column n;
// bias16 = the bias of those columns (shared memory).
__device__ __forceinline__ void gemm_store16(const GemmArgs &a, int row, int n, const uint32_t r[16],
                                             bool split, const float *bias16) {
    if (a.mode == kOutF32) {
        float *crow = a.C + (size_t)row * a.ldc;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            if (n + q >= a.N) break;
            const float v = __uint_as_float(r[q]);
            if (split) atomicAdd(&crow[n + q], v);
            else crow[n + q] = a.accumulate ? crow[n + q] + v : v;
        }
        return;
    }
    float v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        v[q] = __uint_as_float(r[q]) + bias16[q];
        if (a.relu) v[q] = fmaxf(v[q], 0.f);
    }
    if (a.mode == kOutBiasF32) {
        float *yrow = a.C + (size_t)row * a.ldc;
#pragma unroll
        for (int q = 0; q < 16; ++q)
            if (n + q < a.N) yrow[n + q] = v[q];
        return;
    }
    __nv_bfloat16 *yrow = a.y16 + (size_t)row * a.ldc;
    if (n + 16 <= a.N && ((reinterpret_cast<uintptr_t>(yrow + n) & 15u) == 0)) {
        // two 16-byte stores
        uint4 pk[2];
        uint32_t *w = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
            w[q] = *reinterpret_cast<const uint32_t *>(&h2);
        }
        reinterpret_cast<uint4 *>(yrow + n)[0] = pk[0];
        reinterpret_cast<uint4 *>(yrow + n)[1] = pk[1];
    } else {
#pragma unroll
        for (int q = 0; q < 16; ++q)
            if (n + q < a.N) yrow[n + q] = __float2bfloat16(v[q]);
    }
}

template <int BN, int S, bool kAmn, bool kBmn>
__global__ void __launch_bounds__(kGemmThreads, 1)
    gemm_bf16_tc_kernel(const __grid_constant__ CUtensorMap map_a,
                        const __grid_constant__ CUtensorMap map_b,
                        const __grid_constant__ CUtensorMap map_c, GemmArgs a) {
    constexpr uint32_t kStage = (uint32_t)gemm_stage_bytes<BN>();
    static_assert(gemm_smem<BN, S, kAmn || kBmn>() <= 227 * 1024, "stage ring exceeds shared memory");
    static_assert(!(kAmn || kBmn) || BN % 64 == 0, "MN-major operands come in 64-element atoms");
    // the epilogue's staging (4 warps x 32 rows x BN fp32) fits in the ring
    static_assert(S * gemm_stage_bytes<BN>() >= 4 * 32 * BN * 4, "epilogue staging exceeds the ring");
    extern __shared__ uint8_t g_dyn[];
    __shared__ __align__(8) uint64_t s_full[S];
    __shared__ __align__(8) uint64_t s_empty[S];
    __shared__ __align__(8) uint64_t s_done;
    __shared__ uint32_t s_tmem;
    __shared__ float s_bias[BN];  // this tile's bias columns (zero past N)
    // 1024-byte aligned stage buffers (the swizzle atoms)
    const uint32_t base = (smem_addr(g_dyn) + 1023u) & ~1023u;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int m0 = blockIdx.x * kGemmBM, n0 = blockIdx.y * BN;
    const uint32_t done_bar = smem_addr(&s_done);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_addr(&s_tmem)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (t == 0) {
        for (int s = 0; s < S; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_full[s]))
                         : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_empty[s]))
                         : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(done_bar) : "memory");
        // make the initialised barriers visible to the async proxy (TMA,
        // tensor-core commits)
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
        if (a.tma_out)
            asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_c))
                         : "memory");
    }
    if (a.mode != kOutF32)
        for (int c = t; c < BN; c += kGemmThreads) s_bias[c] = n0 + c < a.N ? a.bias[n0 + c] : 0.f;
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    const int kt0 = blockIdx.z * a.ktiles_per;
    const int ktiles = max(0, min(a.ktiles_per, (a.K + kGemmBK - 1) / kGemmBK - kt0));
    const bool split = gridDim.z > 1;

    bool ok = true;
    if (ktiles > 0 && t == 0) {  // producer: TMA loads into the ring
        for (int kt = 0; kt < ktiles; ++kt) {
            const int s = kt % S;
            if (kt >= S &&
                !mbar_wait(smem_addr(&s_empty[s]), (uint32_t)((kt / S - 1) & 1),
                           a.spin_limit)) {
                ok = false;
                break;
            }
            const uint32_t full = smem_addr(&s_full[s]);
            const uint32_t sa = base + (uint32_t)s * kStage, sb = sa + (uint32_t)kGemmATile;
            mbar_arrive_tx(full, kStage);
            const int k = (kt0 + kt) * kGemmBK;
            if (kAmn) {  // two 64-row x 64-column atoms of the stored [K, M]
                tma_load_2d(sa, &map_a, m0, k, full);
                tma_load_2d(sa + 8192u, &map_a, m0 + 64, k, full);
            } else {
                tma_load_2d(sa, &map_a, k, m0, full);
            }
            if (kBmn) {
#pragma unroll
                for (int j = 0; j < BN / 64; ++j)
                    tma_load_2d(sb + (uint32_t)j * 8192u, &map_b, n0 + 64 * j, k, full);
            } else {
                tma_load_2d(sb, &map_b, k, n0, full);
            }
        }
    } else if (ktiles > 0 && t == 32) {  // MMA issuer
        const uint32_t idesc = mma_idesc(kGemmBM, BN, kAmn, kBmn);
        for (int kt = 0; kt < ktiles; ++kt) {
            const int s = kt % S;
            if (!mbar_wait(smem_addr(&s_full[s]), (uint32_t)((kt / S) & 1),
                           a.spin_limit)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sa = base + (uint32_t)s * kStage, sb = sa + (uint32_t)kGemmATile;
#pragma unroll
            for (int ks = 0; ks < kGemmBK / 16; ++ks) {
                const uint64_t ad = kAmn ? smem_desc_sw128_mn(sa + (uint32_t)ks * 2048u)
                                         : smem_desc_sw128(sa + (uint32_t)ks * 32u);
                const uint64_t bd = kBmn ? smem_desc_sw128_mn(sb + (uint32_t)ks * 2048u)
                                         : smem_desc_sw128(sb + (uint32_t)ks * 32u);
                const uint32_t acc = (kt > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            // frees the stage once these MMAs have read it
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    smem_addr(&s_empty[s]))
                : "memory");
        }
        if (ok)
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    done_bar)
                : "memory");
    }
    __syncwarp();
    if (ktiles > 0) ok = mbar_wait(done_bar, 0u, a.spin_limit) && ok;
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    if (!ok) {
        if (t == 0) raise_status(a.status, DEV_LOOKBACK_TIMEOUT);
        // let whatever was issued finish before the CTA's memory goes away
        mbar_wait(done_bar, 0u, a.spin_limit);
    } else if (ktiles > 0 && a.tma_out && (BN >= 64 || a.mode != kOutBiasBF16)) {
        // Every MMA has completed (and so read its stage): the ring holds
        // this warp's 32-row slab, in 128-byte-swizzled boxes of 32 rows x
        // 128 bytes (32 fp32 or 64 bf16 columns) at 4096-byte steps.
        const bool f32 = a.mode != kOutBiasBF16;
        const int box_cols = f32 ? 32 : 64;
        const uint32_t slab = base + (uint32_t)warp * (uint32_t)(32 * BN * (f32 ? 4 : 2));
#pragma unroll 1
        for (int c = 0; c < BN; c += box_cols) {
            const uint32_t box = slab + (uint32_t)(c / box_cols) * 4096u;
            uint32_t r[64];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                if (h * 16 >= box_cols) break;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                    "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
                    : "=r"(r[16 * h + 0]), "=r"(r[16 * h + 1]), "=r"(r[16 * h + 2]),
                      "=r"(r[16 * h + 3]), "=r"(r[16 * h + 4]), "=r"(r[16 * h + 5]),
                      "=r"(r[16 * h + 6]), "=r"(r[16 * h + 7]), "=r"(r[16 * h + 8]),
                      "=r"(r[16 * h + 9]), "=r"(r[16 * h + 10]), "=r"(r[16 * h + 11]),
                      "=r"(r[16 * h + 12]), "=r"(r[16 * h + 13]), "=r"(r[16 * h + 14]),
                      "=r"(r[16 * h + 15])
                    : "r"(lane_addr + (uint32_t)(c + 16 * h))
                    : "memory");
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const uint32_t row_off = (uint32_t)lane * 128u;
            if (f32) {
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    if (a.mode == kOutBiasF32) {
                        float v = __uint_as_float(r[q]) + s_bias[c + q];
                        if (a.relu) v = fmaxf(v, 0.f);
                        r[q] = __float_as_uint(v);
                    }
                }
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    st_shared_v4(box + swz128(row_off + (uint32_t)j * 16u), r[4 * j], r[4 * j + 1],
                                 r[4 * j + 2], r[4 * j + 3]);
            } else {
                uint32_t w[32];
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    float v0 = __uint_as_float(r[2 * q]) + s_bias[c + 2 * q];
                    float v1 = __uint_as_float(r[2 * q + 1]) + s_bias[c + 2 * q + 1];
                    if (a.relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    const __nv_bfloat162 h2 = __floats2bfloat162_rn(v0, v1);
                    w[q] = *reinterpret_cast<const uint32_t *>(&h2);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    st_shared_v4(box + swz128(row_off + (uint32_t)j * 16u), w[4 * j], w[4 * j + 1],
                                 w[4 * j + 2], w[4 * j + 3]);
            }
        }
        // the slab's generic-proxy writes become visible to the tensor store
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncwarp();
        const int y = m0 + warp * 32;
        if (lane == 0 && y < a.M) {
            for (int c = 0; c < BN; c += box_cols) {
                if (n0 + c >= a.N) break;
                const uint32_t box = slab + (uint32_t)(c / box_cols) * 4096u;
                if (split || a.accumulate) tma_reduce_add_2d(&map_c, box, n0 + c, y);
                else tma_store_2d(&map_c, box, n0 + c, y);
            }
            asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
            asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
        }
        __syncwarp();
    } else if (ktiles > 0) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                  "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                  "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(lane_addr + (uint32_t)c)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (row < a.M && n0 + c < a.N) gemm_store16(a, row, n0 + c, r, split, s_bias + c);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"((uint32_t)BN)
                     : "memory");
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// Tensor map of a bf16 operand, 128-byte swizzle, zeros outside.  K-major
// (stored rows x k, ld elements per row): boxes of 64 K-elements x box_rows
// rows.  MN-major (stored k x rows, ld elements per K-row): boxes of 64
// MN-elements x 64 K-rows (one MN atom column of a stage).
static int make_operand_map(CUtensorMap *map, const void *ptr, int rows, int k, int ld,
                            int box_rows, bool mn_major) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return fail(SPLAT_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {mn_major ? (cuuint64_t)rows : (cuuint64_t)k,
                                mn_major ? (cuuint64_t)k : (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2u};
    const cuuint32_t box[2] = {(cuuint32_t)kGemmBK, mn_major ? (cuuint32_t)kGemmBK : (cuuint32_t)box_rows};
    const cuuint32_t elem[2] = {1u, 1u};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims,
                          strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SPLAT_ERR_INVALID_ARG, "tensor map encode failed (%d)", (int)r);
    return SPLAT_OK;
}

// Tensor map of the output (M rows x N columns, ldc elements per row) for the
// epilogue's tensor stores: boxes of 32 rows x 128 bytes (32 fp32 or 64 bf16
// columns), 128-byte swizzle.  Leaves g.tma_out = 0 (register stores) when
// the base or the row stride is not 16-byte aligned.
static int make_output_map(CUtensorMap *map, GemmArgs &g) {
    const bool f32 = g.mode != kOutBiasBF16;
    const void *ptr = f32 ? static_cast<const void *>(g.C) : static_cast<const void *>(g.y16);
    const size_t esize = f32 ? 4 : 2;
    g.tma_out = 0;
    if ((reinterpret_cast<uintptr_t>(ptr) & 15u) || ((size_t)g.ldc * esize) % 16) return SPLAT_OK;
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return fail(SPLAT_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {(cuuint64_t)g.N, (cuuint64_t)g.M};
    const cuuint64_t strides[1] = {(cuuint64_t)g.ldc * esize};
    const cuuint32_t box[2] = {f32 ? 32u : 64u, 32u};
    const cuuint32_t elem[2] = {1u, 1u};
    const CUresult r = fn(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                          2, const_cast<void *>(ptr), dims, strides, box, elem,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SPLAT_ERR_INVALID_ARG, "tensor map encode failed (%d)", (int)r);
    g.tma_out = 1;
    return SPLAT_OK;
}

template <int BN, int S, bool kAmn, bool kBmn>
static int launch_gemm(const CUtensorMap &ma, const CUtensorMap &mb, const CUtensorMap &mc,
                       const GemmArgs &g, dim3 grid, cudaStream_t stream) {
    auto kernel = gemm_bf16_tc_kernel<BN, S, kAmn, kBmn>;
    constexpr int smem = gemm_smem<BN, S, kAmn || kBmn>();
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
        return check_launch("gemm shared-memory attribute");
    kernel<<<grid, kGemmThreads, smem, stream>>>(ma, mb, mc, g);
    return check_launch("gemm_bf16_tc_kernel");
}

// The ring depth follows the K tiles a CTA walks and what shares its SM: 2
// stages when it walks at most 2 (the shared memory left lets more CTAs share
// an SM); 6 (more tensor loads in flight) when that costs no resident CTA --
// 128-column tiles are one per SM at 4 stages already -- or the grid fits
// one wave; else 4, which keeps two 32- or 64-column CTAs per SM.  Measured
// on the network's forward: the first layer (1 K tile) 43.2 -> 31.6 us with
// 2 stages; 128-column layers 20.1 -> 18.4 and 15.4 -> 13.6 us with 6; a
// 64-column layer of 1024 CTAs 30.6 -> 38.6 us with 6, hence 4 there.
template <int BN, bool kAmn, bool kBmn>
static int launch_gemm(const void *A, const void *B, GemmArgs g, int lda, int ldb,
                       cudaStream_t stream) {
    alignas(64) CUtensorMap ma, mb, mc;
    memset(&mc, 0, sizeof(mc));
    if (int rc = make_operand_map(&ma, A, g.M, g.K, lda, kGemmBM, kAmn)) return rc;
    if (int rc = make_operand_map(&mb, B, g.N, g.K, ldb, BN, kBmn)) return rc;
    if (int rc = make_output_map(&mc, g)) return rc;
    const int gm = (g.M + kGemmBM - 1) / kGemmBM, gn = (g.N + BN - 1) / BN;
    const int kt_total = (g.K + kGemmBK - 1) / kGemmBK;
    // split K (kOutF32 only) when the output has few tiles and K is long:
    // partial sums of `ktiles_per` K tiles each are added into C (zeroed
    // first unless accumulating) by tensor reduce-adds (or atomics)
    int splits = 1;
    if (g.mode == kOutF32 && gm * gn < 152 && kt_total >= 16)
        splits = std::min(std::max(1, 2 * 152 / (gm * gn)), kt_total / 8);
    g.ktiles_per = std::max(1, (kt_total + splits - 1) / splits);
    splits = std::max(1, (kt_total + g.ktiles_per - 1) / g.ktiles_per);
    if (splits > 1 && !g.accumulate &&
        cudaMemset2DAsync(g.C, sizeof(float) * (size_t)g.ldc, 0, sizeof(float) * (size_t)g.N,
                          (size_t)g.M, stream) != cudaSuccess)
        return check_launch("gemm split-K zero");
    const dim3 grid(gm, gn, splits);
    if (g.ktiles_per <= 2) return launch_gemm<BN, 2, kAmn, kBmn>(ma, mb, mc, g, grid, stream);
    if (BN == 128 || (long long)gm * gn * splits <= 152)
        return launch_gemm<BN, 6, kAmn, kBmn>(ma, mb, mc, g, grid, stream);
    return launch_gemm<BN, 4, kAmn, kBmn>(ma, mb, mc, g, grid, stream);
}

// Operand rules: 16-byte aligned; K, lda, ldb multiples of 8; a K-major
// operand's leading dimension covers K, an MN-major one's its M (or N).
static int check_operands(const void *A, const void *B, int M, int N, int K, int lda, int ldb,
                          bool a_mn, bool b_mn) {
    if (M < 0 || N < 0 || K < 0) return fail(SPLAT_ERR_INVALID_ARG, "negative GEMM size");
    if (!A || !B) return fail(SPLAT_ERR_INVALID_ARG, "GEMM operand is NULL");
    if (K % 8 || lda % 8 || ldb % 8 || lda < (a_mn ? M : K) || ldb < (b_mn ? N : K))
        return fail(SPLAT_ERR_INVALID_ARG,
                    "GEMM needs K, lda, ldb multiples of 8 (16-byte rows) and lda, ldb covering "
                    "the stored rows");
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) % 16)
        return fail(SPLAT_ERR_INVALID_ARG, "GEMM operands must be 16-byte aligned");
    return SPLAT_OK;
}

static int run_gemm(const void *A, const void *B, GemmArgs g, int lda, int ldb, bool a_mn,
                    bool b_mn, cudaStream_t stream) {
    if (!a_mn && !b_mn) {
        if (g.N <= 32) return launch_gemm<32, false, false>(A, B, g, lda, ldb, stream);
        if (g.N <= 64) return launch_gemm<64, false, false>(A, B, g, lda, ldb, stream);
        return launch_gemm<128, false, false>(A, B, g, lda, ldb, stream);
    }
    // MN-major operands come in 64-element atoms: 64- or 128-column tiles
    const bool narrow = g.N <= 64;
    if (a_mn && b_mn)
        return narrow ? launch_gemm<64, true, true>(A, B, g, lda, ldb, stream)
                      : launch_gemm<128, true, true>(A, B, g, lda, ldb, stream);
    if (a_mn)
        return narrow ? launch_gemm<64, true, false>(A, B, g, lda, ldb, stream)
                      : launch_gemm<128, true, false>(A, B, g, lda, ldb, stream);
    return narrow ? launch_gemm<64, false, true>(A, B, g, lda, ldb, stream)
                  : launch_gemm<128, false, true>(A, B, g, lda, ldb, stream);
}

}  // namespace splat

using namespace splat;

extern "C" {

static int gemm_f32(const void *A, bool a_mn, const void *B, bool b_mn, float *C, int M, int N,
                    int K, int lda, int ldb, int ldc, int accumulate, uint32_t *status_dev,
                    cudaStream_t stream) {
    if (M < 0 || N < 0 || K < 0) return fail(SPLAT_ERR_INVALID_ARG, "negative GEMM size");
    if (M == 0 || N == 0) return SPLAT_OK;
    if (int rc = check_operands(A, B, M, N, K, lda, ldb, a_mn, b_mn)) return rc;
    if (!C || ldc < N) return fail(SPLAT_ERR_INVALID_ARG, "GEMM needs C and ldc >= N");
    if (K == 0) {
        if (accumulate) return SPLAT_OK;
        if (cudaMemset2DAsync(C, sizeof(float) * (size_t)ldc, 0, sizeof(float) * (size_t)N,
                              (size_t)M, stream) != cudaSuccess)
            return check_launch("gemm zero");
        return SPLAT_OK;
    }
    GemmArgs g{};
    g.C = C;
    g.M = M; g.N = N; g.K = K;
    g.ldc = ldc;
    g.accumulate = accumulate;
    g.mode = kOutF32;
    g.status = status_dev;
    g.spin_limit = 1u << 18;  // tries of up to ~1 us each per wait
    return run_gemm(A, B, g, lda, ldb, a_mn, b_mn, stream);
}

int splat_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int lda, int ldb,
                    int ldc, int accumulate, uint32_t *status_dev, splat_stream_t stream) {
    return gemm_f32(A, false, B, false, C, M, N, K, lda, ldb, ldc, accumulate, status_dev,
                    (cudaStream_t)stream);
}

int splat_gemm_bf16_mn(const void *A, int a_mn, const void *B, int b_mn, float *C, int M, int N,
                       int K, int lda, int ldb, int ldc, int accumulate, uint32_t *status_dev,
                       splat_stream_t stream) {
    return gemm_f32(A, a_mn != 0, B, b_mn != 0, C, M, N, K, lda, ldb, ldc, accumulate, status_dev,
                    (cudaStream_t)stream);
}

int splat_gemm_bf16_bias_act(const void *A, const void *B, const float *bias, void *y16,
                             float *y32, int M, int N, int K, int lda, int ldb, int ldy, int relu,
                             uint32_t *status_dev, splat_stream_t stream) {
    if (M < 0 || N < 0 || K < 0) return fail(SPLAT_ERR_INVALID_ARG, "negative GEMM size");
    if (M == 0 || N == 0) return SPLAT_OK;
    if (int rc = check_operands(A, B, M, N, K, lda, ldb, false, false)) return rc;
    if (!bias || (!y16 == !y32) || ldy < N || K == 0)
        return fail(SPLAT_ERR_INVALID_ARG,
                    "GEMM + bias needs K > 0, a bias, exactly one of y16 / y32 and ldy >= N");
    GemmArgs g{};
    g.C = y32;
    g.y16 = static_cast<__nv_bfloat16 *>(y16);
    g.bias = bias;
    g.M = M; g.N = N; g.K = K;
    g.ldc = ldy;
    g.relu = relu;
    g.mode = y16 ? kOutBiasBF16 : kOutBiasF32;
    g.status = status_dev;
    g.spin_limit = 1u << 18;
    return run_gemm(A, B, g, lda, ldb, false, false, (cudaStream_t)stream);
}

}  // extern "C"
