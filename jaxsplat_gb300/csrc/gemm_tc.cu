// gemm_tc.cu -- BF16 GEMM with FP32 accumulation on the 5th-generation tensor
// cores (tcgen05), for the warm-start network's convolutions (as implicit
// im2col GEMMs) and their gradients.
//
//   C[M,N] (fp32, row-major, ldc) (+)= A[M,K] (bf16, row-major: K-major)
//                                       x B[N,K]^T (bf16, row-major: K-major)
//
// One CTA of 128 threads computes a 128 x 128 tile of C.  Operand tiles of
// 128 rows x 64 K-elements are copied into shared memory with cp.async in the
// tensor cores' no-swizzle K-major layout (8-row x 16-byte core matrices;
// the next core matrix along K 128 bytes on, along M/N 1024 bytes on), two
// stages deep.  One thread issues tcgen05.mma (M=128, N=128, K=16, four per
// stage) into a 128-column FP32 accumulator in tensor memory and commits
// each stage to an mbarrier; a stage's buffers are refilled only after that
// barrier flips.  The epilogue reads the accumulator with tcgen05.ld (warp w
// owns TMEM lanes 32w..32w+31 = tile rows) and writes C.
//
// Every wait is bounded: a barrier that does not flip within spin_limit
// polls sets DEV_LOOKBACK_TIMEOUT in the status word, the epilogue is
// skipped, and the CTA frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "splat_internal.cuh"

namespace splat {

constexpr int kGemmBM = 128;
constexpr int kGemmBN = 128;
constexpr int kGemmBK = 64;
constexpr int kGemmThreads = 128;
constexpr int kGemmTileBytes = kGemmBM * kGemmBK * 2;  // 16 KB per operand tile
constexpr int kGemmSmem = 4 * kGemmTileBytes + 1024;   // 2 stages x (A, B) + alignment slack
constexpr uint32_t kGemmTmemCols = 128;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: no swizzle, K-major, leading (K) byte
// offset 128, stride (M/N) byte offset 1024, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

// Polls (non-blocking test_wait) with a short sleep between polls; gives up
// after `limit` polls (about limit x 0.1 us).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (i > 64) __nanosleep(100);
    }
    return false;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}

struct GemmArgs {
    const __nv_bfloat16 *A, *B;
    float *C;
    int M, N, K;
    int lda, ldb, ldc;  // elements
    int accumulate;     // add to C instead of overwriting
    int ktiles_per;     // K tiles per CTA along grid z (split K: partial sums added atomically)
    uint32_t *status;
    uint32_t spin_limit;
};

// Copies the 128 x 64 tile at (row0, k0) of a K-major matrix into the
// core-matrix layout; rows >= rows_total and K past k_total read as zeros.
__device__ __forceinline__ void load_tile(uint32_t sbase, const __nv_bfloat16 *g, int ld,
                                          int row0, int rows_total, int k0, int k_total) {
#pragma unroll
    for (int it = 0; it < (kGemmBM * kGemmBK / 8) / kGemmThreads; ++it) {
        const int q = it * kGemmThreads + threadIdx.x;  // 16-byte chunk index
        const int r = q >> 3, c = q & 7;                // row, chunk along K
        const int row = row0 + r, k = k0 + c * 8;
        const bool ok = row < rows_total && k < k_total;
        const __nv_bfloat16 *src = ok ? g + (size_t)row * ld + k : g;
        const uint32_t dst = sbase + (uint32_t)(((r >> 3) * 8 + c) * 128 + (r & 7) * 16);
        cp_async16(dst, src, ok ? 16u : 0u);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__global__ void __launch_bounds__(kGemmThreads, 1) gemm_bf16_tc_kernel(GemmArgs a) {
    extern __shared__ uint8_t g_dyn[];
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ uint32_t s_tmem;
    // 1024-byte aligned operand area
    const uint32_t raw = smem_addr(g_dyn);
    const uint32_t base = (raw + 1023u) & ~1023u;
    const uint32_t sA[2] = {base, base + kGemmTileBytes};
    const uint32_t sB[2] = {base + 2 * kGemmTileBytes, base + 3 * kGemmTileBytes};
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int m0 = blockIdx.x * kGemmBM, n0 = blockIdx.y * kGemmBN;
    const uint32_t bar0 = smem_addr(&s_bar[0]), bar1 = smem_addr(&s_bar[1]);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_addr(&s_tmem)),
                     "r"(kGemmTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar1) : "memory");
        // make the initialised barriers visible to the tensor cores' arrivals
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = mma_idesc(kGemmBM, kGemmBN);
    const int kt0 = blockIdx.z * a.ktiles_per;
    const int ktiles = max(0, min(a.ktiles_per, (a.K + kGemmBK - 1) / kGemmBK - kt0));
    const bool split = gridDim.z > 1;

    if (ktiles > 0) {
        load_tile(sA[0], a.A, a.lda, m0, a.M, kt0 * kGemmBK, a.K);
        load_tile(sB[0], a.B, a.ldb, n0, a.N, kt0 * kGemmBK, a.K);
    }
    bool ok = true;
    for (int kt = 0; kt < ktiles; ++kt) {
        const int st = kt & 1;
        if (kt + 1 < ktiles) {
            if (kt >= 1) {  // the MMAs of tile kt-1 read the buffers about to be refilled
                const int j = kt - 1;
                const bool done = mbar_wait((j & 1) ? bar1 : bar0, (uint32_t)((j >> 1) & 1),
                                            a.spin_limit);
                if (!__syncthreads_and(done)) {  // a block-uniform decision
                    ok = false;
                    break;
                }
            }
            load_tile(sA[st ^ 1], a.A, a.lda, m0, a.M, (kt0 + kt + 1) * kGemmBK, a.K);
            load_tile(sB[st ^ 1], a.B, a.ldb, n0, a.N, (kt0 + kt + 1) * kGemmBK, a.K);
            asm volatile("cp.async.wait_group 2;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        // the copies were made through the generic proxy; the tensor cores
        // read through the async proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int s = 0; s < kGemmBK / 16; ++s) {
                const uint64_t ad = smem_desc(sA[st] + (uint32_t)s * 256u);
                const uint64_t bd = smem_desc(sB[st] + (uint32_t)s * 256u);
                const uint32_t acc = (kt > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    st ? bar1 : bar0)
                : "memory");
        }
    }
    if (ok && ktiles > 0) {
        const int j = ktiles - 1;
        ok = mbar_wait((j & 1) ? bar1 : bar0, (uint32_t)((j >> 1) & 1), a.spin_limit);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (!ok) {
        if (t == 0) raise_status(a.status, DEV_LOOKBACK_TIMEOUT);
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    } else if (ktiles > 0) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < kGemmBN; c += 16) {
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
            if (row < a.M) {
                float *crow = a.C + (size_t)row * a.ldc;
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int n = n0 + c + q;
                    if (n < a.N) {
                        const float v = __uint_as_float(r[q]);
                        if (split) atomicAdd(&crow[n], v);
                        else crow[n] = a.accumulate ? crow[n] + v : v;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(kGemmTmemCols)
                     : "memory");
    }
}

}  // namespace splat

using namespace splat;

extern "C" {

int splat_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int lda, int ldb,
                    int ldc, int accumulate, uint32_t *status_dev, splat_stream_t stream) {
    if (M < 0 || N < 0 || K < 0) return fail(SPLAT_ERR_INVALID_ARG, "negative GEMM size");
    if (M == 0 || N == 0) return SPLAT_OK;
    if (!A || !B || !C) return fail(SPLAT_ERR_INVALID_ARG, "GEMM operand is NULL");
    if (K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N)
        return fail(SPLAT_ERR_INVALID_ARG,
                    "GEMM needs K, lda, ldb multiples of 8 (16-byte rows), lda, ldb >= K, ldc >= N");
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) % 16)
        return fail(SPLAT_ERR_INVALID_ARG, "GEMM operands must be 16-byte aligned");
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(gemm_bf16_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kGemmSmem) != cudaSuccess)
            return check_launch("gemm shared-memory attribute");
        attr_set = true;
    }
    GemmArgs g;
    g.A = static_cast<const __nv_bfloat16 *>(A);
    g.B = static_cast<const __nv_bfloat16 *>(B);
    g.C = C;
    g.M = M; g.N = N; g.K = K;
    g.lda = lda; g.ldb = ldb; g.ldc = ldc;
    g.accumulate = accumulate;
    g.status = status_dev;
    g.spin_limit = 1u << 21;  // ~0.2 s of polling per wait
    // split K when the output has few tiles and K is long: partial sums of
    // `ktiles_per` K tiles each are added atomically into C (zeroed first
    // unless accumulating)
    const int gm = (M + kGemmBM - 1) / kGemmBM, gn = (N + kGemmBN - 1) / kGemmBN;
    const int kt_total = (K + kGemmBK - 1) / kGemmBK;
    int splits = 1;
    if (gm * gn < 152 && kt_total >= 16)
        splits = std::min(std::max(1, 2 * 152 / (gm * gn)), kt_total / 8);
    g.ktiles_per = std::max(1, (kt_total + splits - 1) / splits);
    splits = std::max(1, (kt_total + g.ktiles_per - 1) / g.ktiles_per);
    if (K == 0) {
        if (accumulate) return SPLAT_OK;
        if (cudaMemset2DAsync(C, sizeof(float) * (size_t)ldc, 0, sizeof(float) * (size_t)N,
                              (size_t)M, (cudaStream_t)stream) != cudaSuccess)
            return check_launch("gemm zero");
        return SPLAT_OK;
    }
    if (splits > 1 && !accumulate &&
        cudaMemset2DAsync(C, sizeof(float) * (size_t)ldc, 0, sizeof(float) * (size_t)N, (size_t)M,
                          (cudaStream_t)stream) != cudaSuccess)
        return check_launch("gemm split-K zero");
    dim3 grid(gm, gn, splits);
    gemm_bf16_tc_kernel<<<grid, kGemmThreads, kGemmSmem, (cudaStream_t)stream>>>(g);
    return check_launch("gemm_bf16_tc_kernel");
}

}  // extern "C"
