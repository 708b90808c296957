// sort.cu -- intersection key emission, stable onesweep LSD radix sort of the
// 64-bit tile|depth keys, and tile bin edges.
//
// Output contract (lib/ops.cu:645-793): gaussian_ids_sorted is the stable
// ascending order of the keys over bits [0, end_bit), end_bit = 32 + msb with
// msb = bitlength(T) + 1 (lib/ops.cu:723-724); ties keep emission order.
// tile_bins[t] = [first, last+1) of tile t in that order, (0,0) when empty.
//
// Radix sort: one histogram pass over the keys computes the digit counts of
// every 8-bit digit position at once; then one "onesweep" kernel per digit
// position (Adinets & Merrill, "Onesweep: A Faster Least Significant Digit
// Radix Sort for GPUs", 2022): each block takes a 3072-key partition by
// ticket, ranks its keys stably with warp match/popc, publishes its per-digit
// counts, resolves their global offsets with a decoupled look-back over the
// preceding partitions and scatters keys+ids through shared memory, so every
// pass reads and writes each key once.
#include "splat_internal.cuh"
#include "splat_math.cuh"

namespace splat {

// ---------------------------------------------------------------------------
// Key emission (forward.cu:135-179).  A block owns 256 consecutive Gaussians;
// their tile rectangles are expanded cooperatively so that consecutive
// threads write consecutive slots (the reference loops per thread over the
// rectangle, which serialises large Gaussians and scatters the writes).

constexpr int kEmitBlock = 256;

struct EmitArgs {
    int n;
    const float *xys, *depths;
    const int32_t *radii, *cum;
    unsigned tiles_x, tiles_y, bw;
    long long count;
    unsigned long long *keys;
    int32_t *ids;
    uint32_t *status;
};

__global__ void __launch_bounds__(kEmitBlock) emit_kernel(EmitArgs a) {
    __shared__ int s_off[kEmitBlock + 1];  // block-local exclusive offsets
    __shared__ int s_start[kEmitBlock];    // global first slot (cum[g-1])
    __shared__ unsigned s_x0[kEmitBlock], s_y0[kEmitBlock], s_w[kEmitBlock];
    __shared__ int s_dbits[kEmitBlock];
    const int t = threadIdx.x;
    const int g = blockIdx.x * kEmitBlock + t;
    int cnt = 0;
    if (g < a.n) {
        const int rad = a.radii[g];
        if (rad > 0) {
            const float2 c = make_float2(a.xys[2 * g], a.xys[2 * g + 1]);
            const TileRect r = tile_rect(c, (float)rad, a.tiles_x, a.tiles_y, a.bw);
            s_x0[t] = r.x0;
            s_y0[t] = r.y0;
            s_w[t] = r.x1 - r.x0;
            cnt = (int)((r.x1 - r.x0) * (r.y1 - r.y0));
            s_dbits[t] = __float_as_int(a.depths[g]);
        }
        s_start[t] = g == 0 ? 0 : a.cum[g - 1];
    }
    // block exclusive scan of cnt
    const int lane = t & 31, warp = t >> 5;
    int v = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    __shared__ int s_warp[kEmitBlock / 32];
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int w = 0; w < kEmitBlock / 32; ++w) {
            const int x = s_warp[w];
            s_warp[w] = run;
            run += x;
        }
        s_off[kEmitBlock] = run;
    }
    __syncthreads();
    s_off[t] = s_warp[warp] + v - cnt;
    __syncthreads();
    const int total = s_off[kEmitBlock];
    for (int s = t; s < total; s += kEmitBlock) {
        // owner: last j with s_off[j] <= s (skips Gaussians with no slots)
        int lo = 0, hi = kEmitBlock - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_off[mid] <= s) lo = mid; else hi = mid - 1;
        }
        const int j = lo;
        const int k = s - s_off[j];
        const unsigned w = s_w[j];
        const unsigned ty = s_y0[j] + (unsigned)k / w;
        const unsigned tx = s_x0[j] + (unsigned)k % w;
        const long long slot = (long long)s_start[j] + k;
        if (slot < 0 || slot >= a.count) {
            raise_status(a.status, DEV_EMIT_OVERFLOW);
            continue;
        }
        const unsigned long long tile = (unsigned long long)(ty * a.tiles_x + tx);
        const unsigned long long key = (tile << 32) | (unsigned long long)(long long)s_dbits[j];
        a.keys[slot] = key;
        a.ids[slot] = blockIdx.x * kEmitBlock + j;
    }
}

// ---------------------------------------------------------------------------
// Radix sort.

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kMaxPasses = 8;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 12;
constexpr int kPartKeys = kSortThreads * kSortItems;  // 3072 keys per partition
constexpr int kHistCopies = 4;

__device__ __forceinline__ unsigned digit_of(unsigned long long key, int shift, unsigned mask) {
    return (unsigned)(key >> shift) & mask;
}

struct HistArgs {
    const unsigned long long *keys;
    long long count;
    int passes;
    int end_bit;
    unsigned *hist;  // [passes][256]
};

__global__ void __launch_bounds__(256) radix_hist_kernel(HistArgs a) {
    __shared__ unsigned sh[kHistCopies][kMaxPasses][kRadix];
    for (int i = threadIdx.x; i < kHistCopies * kMaxPasses * kRadix; i += blockDim.x)
        (&sh[0][0][0])[i] = 0u;
    __syncthreads();
    const int copy = (threadIdx.x >> 5) & (kHistCopies - 1);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += stride) {
        const unsigned long long k = a.keys[i];
        for (int d = 0; d < a.passes; ++d) {
            const int shift = d * kRadixBits;
            const int bits = min(kRadixBits, a.end_bit - shift);
            atomicAdd(&sh[copy][d][digit_of(k, shift, (1u << bits) - 1u)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < a.passes * kRadix; i += blockDim.x) {
        unsigned s = 0;
#pragma unroll
        for (int c = 0; c < kHistCopies; ++c) s += sh[c][i / kRadix][i % kRadix];
        if (s) atomicAdd(&a.hist[i], s);
    }
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void __launch_bounds__(kRadix) radix_offsets_kernel(const unsigned *hist, unsigned *offs) {
    __shared__ unsigned s[kRadix];
    const int d = blockIdx.x, t = threadIdx.x;
    const unsigned x = hist[d * kRadix + t];
    s[t] = x;
    __syncthreads();
    for (int o = 1; o < kRadix; o <<= 1) {
        const unsigned y = t >= o ? s[t - o] : 0u;
        __syncthreads();
        s[t] += y;
        __syncthreads();
    }
    offs[d * kRadix + t] = s[t] - x;
}

// 32-bit look-back words: [flag:2][count:30].
constexpr uint32_t kLbAgg = 1u << 30;
constexpr uint32_t kLbPrefix = 2u << 30;
constexpr uint32_t kLbMask = (1u << 30) - 1u;

__device__ __forceinline__ uint32_t wait_word(uint32_t *slot, uint32_t limit, uint32_t *status) {
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> a(*slot);
    for (uint32_t i = 0; i < limit; ++i) {
        const uint32_t w = a.load(cuda::memory_order_acquire);
        if (w & (kLbAgg | kLbPrefix)) return w;
        if (i > 32) __nanosleep(64);
    }
    raise_status(status, DEV_LOOKBACK_TIMEOUT);
    return kLbPrefix;
}

__device__ __forceinline__ void publish_word(uint32_t *slot, uint32_t w) {
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> a(*slot);
    a.store(w, cuda::memory_order_release);
}

struct PassArgs {
    const unsigned long long *keys_in;
    const int32_t *vals_in;
    unsigned long long *keys_out;
    int32_t *vals_out;
    long long count;
    int shift;
    unsigned mask;
    const unsigned *offs;  // [256] exclusive global digit offsets of this pass
    uint32_t *lookback;    // [nparts][256]
    unsigned *ticket;
    uint32_t *status;
    uint32_t spin_limit;
};

__global__ void __launch_bounds__(kSortThreads) onesweep_kernel(PassArgs a) {
    __shared__ unsigned s_whist[kSortWarps][kRadix];  // per-warp digit counts -> exclusive offsets
    __shared__ unsigned s_bstart[kRadix];             // block-local digit start
    __shared__ unsigned s_gbase[kRadix];              // global position of the block's first key of digit
    __shared__ unsigned long long s_keys[kPartKeys];
    __shared__ int32_t s_vals[kPartKeys];
    __shared__ int s_part;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_part = (int)atomicAdd(a.ticket, 1u);
    for (int i = lane; i < kRadix; i += 32) s_whist[warp][i] = 0u;
    __syncthreads();
    const int part = s_part;
    const long long base = (long long)part * kPartKeys + (long long)warp * 32 * kSortItems;

    unsigned long long key[kSortItems];
    int32_t val[kSortItems];
    unsigned rank[kSortItems];
    unsigned dig[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const long long idx = base + k * 32 + lane;
        const bool ok = idx < a.count;
        key[k] = ok ? a.keys_in[idx] : 0ull;
        val[k] = ok ? a.vals_in[idx] : 0;
        dig[k] = ok ? digit_of(key[k], a.shift, a.mask) : (unsigned)kRadix;  // kRadix = absent
    }
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const unsigned d = dig[k];
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned before = s_whist[warp][d & (kRadix - 1)];
        __syncwarp();
        rank[k] = before + __popc(peers & lt_mask);
        if (d < (unsigned)kRadix && lane == __ffs(peers) - 1) s_whist[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // per digit (thread t = digit t): warp offsets, block count, look-back
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        const unsigned c = s_whist[w][t];
        s_whist[w][t] = run;
        run += c;
    }
    const unsigned cnt = run;
    uint32_t *my = a.lookback + (size_t)part * kRadix + t;
    unsigned excl = 0;
    if (part == 0) {
        publish_word(my, kLbPrefix | (cnt & kLbMask));
    } else {
        publish_word(my, kLbAgg | (cnt & kLbMask));
        for (int j = part - 1; j >= 0; --j) {
            const uint32_t w = wait_word(a.lookback + (size_t)j * kRadix + t, a.spin_limit, a.status);
            excl += w & kLbMask;
            if (w & kLbPrefix) break;
        }
        publish_word(my, kLbPrefix | ((excl + cnt) & kLbMask));
    }
    s_gbase[t] = a.offs[t] + excl;
    // block-local exclusive scan of the digit counts (for staging)
    s_bstart[t] = cnt;
    __syncthreads();
    for (int o = 1; o < kRadix; o <<= 1) {
        const unsigned y = t >= o ? s_bstart[t - o] : 0u;
        __syncthreads();
        s_bstart[t] += y;
        __syncthreads();
    }
    const unsigned bstart = s_bstart[t] - cnt;
    __syncthreads();
    s_bstart[t] = bstart;
    __syncthreads();

    // stage in digit order
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const unsigned d = dig[k];
        if (d < (unsigned)kRadix) {
            const unsigned pos = s_bstart[d] + s_whist[warp][d] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = val[k];
        }
    }
    __syncthreads();
    const long long remaining = a.count - (long long)part * kPartKeys;
    const int nvalid = remaining < kPartKeys ? (int)remaining : kPartKeys;
    for (int i = t; i < nvalid; i += kSortThreads) {
        const unsigned long long k = s_keys[i];
        const unsigned d = digit_of(k, a.shift, a.mask);
        const long long g = (long long)s_gbase[d] + (i - (int)s_bstart[d]);
        if (g < 0 || g >= a.count) {
            raise_status(a.status, DEV_SORT_OVERFLOW);
            continue;
        }
        a.keys_out[g] = k;
        a.vals_out[g] = s_vals[i];
    }
}

// ---------------------------------------------------------------------------
// Tile bin edges: one thread per tile, binary search of the tile field of the
// sorted keys (masked to the sorted bits).  Writes every tile, (0,0) when
// empty, so no zeroing pass is needed (the reference memsets then marks the
// boundaries, forward.cu:184-208).

struct BinArgs {
    const unsigned long long *keys;
    long long count;
    unsigned long long mask;
    int ntiles;
    int2 *bins;
};

__device__ __forceinline__ long long lower_tile(const BinArgs &a, unsigned long long tile) {
    long long lo = 0, hi = a.count;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (((a.keys[mid] & a.mask) >> 32) < tile) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void tile_bins_kernel(BinArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.ntiles) return;
    const long long lo = lower_tile(a, (unsigned long long)t);
    const long long hi = lower_tile(a, (unsigned long long)t + 1);
    a.bins[t] = lo < hi ? make_int2((int)lo, (int)hi) : make_int2(0, 0);
}

// ---------------------------------------------------------------------------
// Host side.

int sort_end_bit(unsigned ntiles) {
    int bits = 0;
    while ((ntiles >> bits) != 0) ++bits;  // 32 - clz(T)
    return 32 + bits + 1;
}

struct SortLayout {
    unsigned long long *keys_a, *keys_b;
    int32_t *vals_a, *vals_b;
    unsigned *hist, *offs, *tickets;
    uint32_t *lookback;
    size_t zero_bytes;  // hist + tickets + lookback are contiguous from `hist`
};

static SortLayout sort_layout(Arena &ar, long long count, int passes) {
    SortLayout L;
    const long long nparts = (count + kPartKeys - 1) / kPartKeys;
    L.keys_a = ar.take<unsigned long long>(count);
    L.keys_b = ar.take<unsigned long long>(count);
    L.vals_a = ar.take<int32_t>(count);
    L.vals_b = ar.take<int32_t>(count);
    L.offs = ar.take<unsigned>((size_t)passes * kRadix);
    const size_t before = (ar.used + 255) & ~size_t(255);
    L.hist = ar.take<unsigned>((size_t)passes * kRadix);
    L.tickets = ar.take<unsigned>(kMaxPasses);
    L.lookback = ar.take<uint32_t>((size_t)passes * nparts * kRadix);
    L.zero_bytes = ar.used - before;
    return L;
}

size_t sort_workspace_bytes(const splat_params &p, long long count) {
    const int passes = (sort_end_bit(n_tiles(p)) + kRadixBits - 1) / kRadixBits;
    Arena ar{nullptr, 0};
    sort_layout(ar, count, passes);
    return ar.used + 256;
}

int launch_sort_and_bin(const splat_params &p, long long count, const float *xys,
                        const float *depths, const int32_t *radii, const int32_t *cum,
                        int32_t *ids_sorted, int2 *bins, long long *isect_out,
                        int32_t *ids_unsorted_out, long long *keys_sorted_out, void *ws,
                        size_t ws_bytes, cudaStream_t s) {
    const unsigned tx = tiles_x(p), ty = tiles_y(p), T = tx * ty;
    const int end_bit = sort_end_bit(T);
    const int passes = (end_bit + kRadixBits - 1) / kRadixBits;
    Arena ar{static_cast<char *>(ws), ws_bytes};
    SortLayout L = sort_layout(ar, count, passes);
    if (!ar.fits())
        return fail(SPLAT_ERR_WORKSPACE, "sort workspace too small: need %zu bytes, got %zu",
                    ar.used, ws_bytes);
    if (count == 0) {
        if (cudaMemsetAsync(bins, 0, sizeof(int2) * T, s) != cudaSuccess)
            return check_launch("tile_bins memset");
        return SPLAT_OK;
    }
    // emission
    {
        EmitArgs e;
        e.n = (int)p.num_points;
        e.xys = xys; e.depths = depths; e.radii = radii; e.cum = cum;
        e.tiles_x = tx; e.tiles_y = ty; e.bw = p.block_width;
        e.count = count;
        e.keys = L.keys_a;
        e.ids = L.vals_a;
        e.status = p.device_status;
        emit_kernel<<<(e.n + kEmitBlock - 1) / kEmitBlock, kEmitBlock, 0, s>>>(e);
        if (int rc = check_launch("emit_kernel")) return rc;
    }
    if (isect_out && cudaMemcpyAsync(isect_out, L.keys_a, sizeof(long long) * count,
                                     cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return check_launch("isect_ids copy");
    if (ids_unsorted_out && cudaMemcpyAsync(ids_unsorted_out, L.vals_a, sizeof(int32_t) * count,
                                            cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return check_launch("gaussian_ids copy");
    if (cudaMemsetAsync(L.hist, 0, L.zero_bytes, s) != cudaSuccess)
        return check_launch("sort workspace memset");
    {
        HistArgs h{L.keys_a, count, passes, end_bit, L.hist};
        long long blocks = (count + 256 * 16 - 1) / (256 * 16);
        if (blocks > 152 * 8) blocks = 152 * 8;
        radix_hist_kernel<<<(unsigned)blocks, 256, 0, s>>>(h);
        if (int rc = check_launch("radix_hist_kernel")) return rc;
        radix_offsets_kernel<<<passes, kRadix, 0, s>>>(L.hist, L.offs);
        if (int rc = check_launch("radix_offsets_kernel")) return rc;
    }
    const long long nparts = (count + kPartKeys - 1) / kPartKeys;
    unsigned long long *kin = L.keys_a, *kout = L.keys_b;
    int32_t *vin = L.vals_a, *vout = L.vals_b;
    for (int d = 0; d < passes; ++d) {
        const bool last = d == passes - 1;
        PassArgs pa;
        pa.keys_in = kin;
        pa.vals_in = vin;
        pa.keys_out = kout;
        pa.vals_out = last ? ids_sorted : vout;
        pa.count = count;
        pa.shift = d * kRadixBits;
        pa.mask = (1u << min(kRadixBits, end_bit - d * kRadixBits)) - 1u;
        pa.offs = L.offs + d * kRadix;
        pa.lookback = L.lookback + (size_t)d * nparts * kRadix;
        pa.ticket = L.tickets + d;
        pa.status = p.device_status;
        pa.spin_limit = spin_limit(p);
        onesweep_kernel<<<(unsigned)nparts, kSortThreads, 0, s>>>(pa);
        if (int rc = check_launch("onesweep_kernel")) return rc;
        unsigned long long *tk = kin; kin = kout; kout = tk;
        int32_t *tv = vin; vin = vout; vout = tv;
    }
    // kin now holds the sorted keys
    if (keys_sorted_out && cudaMemcpyAsync(keys_sorted_out, kin, sizeof(long long) * count,
                                           cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return check_launch("isect_ids_sorted copy");
    BinArgs b;
    b.keys = kin;
    b.count = count;
    b.mask = end_bit >= 64 ? ~0ull : ((1ull << end_bit) - 1ull);
    b.ntiles = (int)T;
    b.bins = bins;
    tile_bins_kernel<<<(T + 255) / 256, 256, 0, s>>>(b);
    return check_launch("tile_bins_kernel");
}

}  // namespace splat
