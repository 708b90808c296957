// sort.cu -- intersection ordering: depth sort of the Gaussians, tile-key
// emission, stable tile sort, tile bin edges.
//
// Output contract (lib/ops.cu:645-793): gaussian_ids_sorted is the stable
// ascending order of the keys (tile << 32 | depth_bits) over bits
// [0, end_bit), end_bit = 32 + bitlength(T) + 1 (lib/ops.cu:723-724), of the
// reference's emission order (Gaussian index, then row-major tile); so within
// a tile, entries are ordered by depth bits and ties by Gaussian index.
// tile_bins[t] = [first, last + 1) of tile t in that order, (0, 0) when empty.
//
// How it is produced here (same order, a quarter of the memory traffic of a
// 6-pass sort of 12-byte pairs):
//  1. the N Gaussians are sorted by their 32-bit depth bits (stable, so equal
//     depths stay in index order; Gaussians that hit no tile sort last);
//  2. intersections are emitted in that depth order: (tile id, Gaussian id)
//     pairs of 4 + 4 bytes, each block finding its output offset with a
//     decoupled look-back over the preceding blocks' counts;
//  3. the pairs are sorted stably by tile id alone (ceil(bitlength(T-1) / 8)
//     passes: 2 at 1920x1080) -- stability keeps the depth order inside a
//     tile;
//  4. bin edges come from a binary search per tile.
// Sorting uses an in-house onesweep LSD radix sort (Adinets & Merrill,
// "Onesweep: A Faster Least Significant Digit Radix Sort for GPUs", 2022):
// the digit counts of every pass come from the kernel that writes the keys
// (or one histogram pass); each pass is one kernel in which a block takes a
// 4096-key partition by ticket, ranks its keys stably with per-bit warp
// ballots and popc, publishes its per-digit counts, resolves their global
// offsets by a decoupled look-back over preceding partitions (plus the
// pass's digit starts, scanned from the counts by every block) and scatters
// through shared memory.
#include <algorithm>

#include "splat_internal.cuh"
#include "splat_math.cuh"

namespace splat {

// ---------------------------------------------------------------------------
// Onesweep radix sort of 32-bit keys with 32-bit values.

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kMaxPasses = 4;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kPartKeys = kSortThreads * kSortItems;  // 4096 keys per partition
constexpr int kHistCopies = 4;

__device__ __forceinline__ unsigned digit_of(uint32_t key, int shift, unsigned mask) {
    return (key >> shift) & mask;
}

struct HistArgs {
    const uint32_t *keys;
    Count count;
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
    const long long count = a.count.get();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const uint32_t k = a.keys[i];
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

// Digit counts of the keys a producer kernel writes, for every pass of the
// radix sort that follows (the sort then skips its histogram pass over the
// keys): a block counts in shared memory and adds its nonzero counts to the
// global histogram once.
struct KeyHist {
    unsigned *hist;  // [passes][kRadix] of the sort, zeroed before the producer; null: none
    int passes;
    int end_bit;
};

__device__ __forceinline__ void key_hist_zero(unsigned (*sh)[kRadix]) {
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) (&sh[0][0])[i] = 0u;
}

__device__ __forceinline__ void key_hist_add(const KeyHist &h, unsigned (*sh)[kRadix], uint32_t k) {
    for (int d = 0; d < h.passes; ++d) {
        const int shift = d * kRadixBits;
        const int bits = min(kRadixBits, h.end_bit - shift);
        atomicAdd(&sh[d][digit_of(k, shift, (1u << bits) - 1u)], 1u);
    }
}

__device__ __forceinline__ void key_hist_flush(const KeyHist &h, unsigned (*sh)[kRadix]) {
    for (int i = threadIdx.x; i < h.passes * kRadix; i += blockDim.x) {
        const unsigned c = (&sh[0][0])[i];
        if (c) atomicAdd(&h.hist[i], c);
    }
}

// 32-bit look-back words: [flag:2][count:30].  The count travels inside the
// word, so the words need no ordering against other memory: relaxed loads and
// stores at device scope are enough.
constexpr uint32_t kLbAgg = 1u << 30;
constexpr uint32_t kLbPrefix = 2u << 30;
constexpr uint32_t kLbMask = (1u << 30) - 1u;
// Predecessor words read at once per look-back step.  The walk back to the
// nearest published prefix is a chain of dependent L2 round trips; reading a
// window of them together shortens the chain by the window's length.
constexpr int kLbWindow = 8;

__device__ __forceinline__ uint32_t load_word(const uint32_t *slot) {
    cuda::atomic_ref<const uint32_t, cuda::thread_scope_device> a(*slot);
    return a.load(cuda::memory_order_relaxed);
}

__device__ __forceinline__ uint32_t wait_word(const uint32_t *slot, uint32_t limit, uint32_t *status) {
    for (uint32_t i = 0; i < limit; ++i) {
        const uint32_t w = load_word(slot);
        if (w & (kLbAgg | kLbPrefix)) return w;
        if (i > 32) __nanosleep(64);
    }
    raise_status(status, DEV_LOOKBACK_TIMEOUT);
    return kLbPrefix;
}

__device__ __forceinline__ void publish_word(uint32_t *slot, uint32_t w) {
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> a(*slot);
    a.store(w, cuda::memory_order_relaxed);
}

// Exclusive prefix of one digit for partition `part` (> 0): the words of
// partitions part-1, part-2, ... (stride `stride` words apart) are summed
// down to and including the nearest one flagged as an inclusive prefix.
__device__ __forceinline__ unsigned lookback_digit(const uint32_t *words, size_t stride, int part,
                                                   uint32_t limit, uint32_t *status) {
    unsigned excl = 0;
    bool done = false;
    for (int j = part - 1; !done; j -= kLbWindow) {
        uint32_t w[kLbWindow];
#pragma unroll
        for (int i = 0; i < kLbWindow; ++i)
            w[i] = j - i >= 0 ? load_word(words + (size_t)(j - i) * stride) : kLbPrefix;
#pragma unroll
        for (int i = 0; i < kLbWindow; ++i) {
            if (!done) {
                uint32_t x = w[i];
                // j - i >= 0 here: partition 0 publishes a prefix, so the walk
                // stops there at the latest
                if (!(x & (kLbAgg | kLbPrefix)))
                    x = wait_word(words + (size_t)(j - i) * stride, limit, status);
                excl += x & kLbMask;
                done = (x & kLbPrefix) != 0;
            }
        }
    }
    return excl;
}

// Lanes of the warp whose digit d equals this lane's, over the low `nbits`
// bits: one ballot per digit bit (a lane keeps the ballot where its own bit is
// set, the complement where it is clear).  Measured faster than match.any
// (sort stage 0.336 vs 0.360 ms at 1080p, 2.98 vs 3.32 ms at 4K): match.any
// slows down with the number of distinct digits in the warp, and the low
// digit of a tile id or depth is nearly distinct across 32 lanes.
__device__ __forceinline__ unsigned match_digit(unsigned d, int nbits) {
    unsigned peers = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < kRadixBits; ++b) {
        if (b < nbits) {
            const unsigned bit = (d >> b) & 1u;
            const unsigned m = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? m : ~m;
        }
    }
    return peers;
}

struct PassArgs {
    const uint32_t *keys_in;
    const int32_t *vals_in;
    uint32_t *keys_out;
    int32_t *vals_out;
    Count count;
    int shift;
    unsigned mask;
    const unsigned *hist;  // [256] global digit counts of this pass (complete before the pass)
    uint32_t *lookback;    // [nparts][256]
    unsigned *ticket;
    uint32_t *status;
    uint32_t spin_limit;
};

__global__ void __launch_bounds__(kSortThreads, 4) onesweep_kernel(PassArgs a) {
    __shared__ unsigned s_whist[kSortWarps][kRadix];  // per-warp digit counts -> exclusive offsets
    __shared__ int s_delta[kRadix];                   // block-local digit start, then global - local
    __shared__ unsigned s_wsum[kSortWarps];
    __shared__ unsigned s_hsum[kSortWarps];
    __shared__ unsigned s_hc[kRadix];  // this pass's global digit counts
    __shared__ uint32_t s_keys[kPartKeys];
    __shared__ int32_t s_vals[kPartKeys];
    __shared__ int s_part;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_part = (int)atomicAdd(a.ticket, 1u);
    for (int i = lane; i < kRadix; i += 32) s_whist[warp][i] = 0u;
    // this pass's global count of digit t: every block scans the 256 counts
    // itself (their exclusive prefix is the digit's first output slot), so
    // no separate offsets kernel runs between the producer and the pass.
    // Parked in shared memory until the scan (no register across the ranking).
    s_hc[t] = a.hist[t];
    __syncthreads();
    const int part = s_part;
    // counts are at most 2^30 - 1 (checked on the host), so 32-bit indices
    const int count = (int)a.count.get();
    if (part * kPartKeys >= count) return;  // past the end (capacity-sized grid)
    // warp-striped: warp w owns keys [base, base + 32*items), item k of lane l
    // is key base + 32k + l, so (k, l) order is key order
    const int base = part * kPartKeys + warp * 32 * kSortItems + lane;
    // the partition's values are read only after the ranking: start bringing
    // them into L2 now (whole 16-byte chunks, from a 16-byte aligned start:
    // partitions are 16 KB apart, so only the buffer's own alignment matters)
    if (t == 0) {
        const int32_t *src = a.vals_in + (size_t)part * kPartKeys;
        const uint32_t bytes = (uint32_t)(min(count - part * kPartKeys, kPartKeys) * 4) & ~15u;
        if (bytes && (reinterpret_cast<uintptr_t>(src) & 15u) == 0)
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes)
                         : "memory");
    }

    uint32_t key[kSortItems];
    unsigned rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) key[k] = base + k * 32 < count ? a.keys_in[base + k * 32] : 0u;
    // Stable rank of each key among the warp's keys with the same digit:
    // the lanes holding a digit (match_digit) are ranked by lane, and the
    // lowest of them adds their number to the warp's digit counter.  The
    // counter updates of successive items are shared-memory atomics issued
    // in item order, so they need no barrier between items and overlap.
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nbits = __popc(a.mask);
    const bool full = (part + 1) * kPartKeys <= count;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const bool ok = base + k * 32 < count;
        const unsigned d = ok ? digit_of(key[k], a.shift, a.mask) : 0u;
        // past the end only in the last partition: those lanes join no group
        const unsigned peers = match_digit(d, nbits) & (full ? 0xffffffffu : __ballot_sync(0xffffffffu, ok));
        const int leader = __ffs(peers) - 1;
        unsigned before = 0;
        if (ok && lane == leader) before = atomicAdd(&s_whist[warp][d], (unsigned)__popc(peers));
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[k] = ok ? before + __popc(peers & lt_mask) : 0xffffffffu;
    }
    __syncthreads();

    // per digit (thread t = digit t): warp offsets, block count
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        const unsigned c = s_whist[w][t];
        s_whist[w][t] = run;
        run += c;
    }
    const unsigned cnt = run;
    uint32_t *my = a.lookback + (size_t)part * kRadix + t;
    publish_word(my, (part == 0 ? kLbPrefix : kLbAgg) | (cnt & kLbMask));
    // block-local exclusive scan of the digit counts: warp scans + warp totals
    unsigned incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    unsigned wbase = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) wbase += w < warp ? s_wsum[w] : 0u;
    const unsigned bstart = wbase + incl - cnt;
    s_delta[t] = (int)bstart;
    __syncthreads();

    // stage in digit order; the values are loaded only now (coalesced, in
    // key order) so that they take no registers during the ranking
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        if (rank[k] != 0xffffffffu) {
            const unsigned d = digit_of(key[k], a.shift, a.mask);
            rank[k] += (unsigned)s_delta[d] + s_whist[warp][d];
            if (rank[k] < (unsigned)kPartKeys) s_keys[rank[k]] = key[k];
        }
    }
#pragma unroll
    for (int k = 0; k < kSortItems; ++k)
        if (rank[k] < (unsigned)kPartKeys) s_vals[rank[k]] = a.vals_in[base + k * 32];
    // look-back last, after the staging: the predecessors have had that long
    // to publish their prefixes, and the keys are out of registers
    unsigned excl = 0;
    if (part > 0) {
        excl = lookback_digit(a.lookback + t, kRadix, part, a.spin_limit, a.status);
        publish_word(my, kLbPrefix | ((excl + cnt) & kLbMask));
    }
    // the pass's global digit offsets: exclusive scan of its digit counts
    const unsigned hc = s_hc[t];
    unsigned hincl = hc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned hy = __shfl_up_sync(0xffffffffu, hincl, o);
        if (lane >= o) hincl += hy;
    }
    if (lane == 31) s_hsum[warp] = hincl;
    __syncthreads();  // every thread has read s_delta for its staging; s_hsum is complete
    unsigned hbase = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) hbase += w < warp ? s_hsum[w] : 0u;
    const unsigned goff = hbase + hincl - hc;  // first global slot of digit t
    // staged position i of digit d goes to global position i + delta[d]
    s_delta[t] = (int)(goff + excl) - (int)bstart;
    __syncthreads();
    const int nvalid = min(count - part * kPartKeys, kPartKeys);
#pragma unroll 4
    for (int i = t; i < nvalid; i += kSortThreads) {
        const uint32_t k = s_keys[i];
        const int g = s_delta[digit_of(k, a.shift, a.mask)] + i;
        if ((unsigned)g >= (unsigned)count) {
            raise_status(a.status, DEV_SORT_OVERFLOW);
            continue;
        }
        a.keys_out[g] = k;
        a.vals_out[g] = s_vals[i];
    }
}

struct RadixBufs {
    uint32_t *ka, *kb;
    int32_t *va, *vb;
    unsigned *hist, *tickets;
    uint32_t *lookback;
    size_t zero_bytes;  // hist + tickets + lookback, contiguous from hist
    long long nparts;
    int passes;
};

static RadixBufs radix_layout(Arena &ar, long long count, int end_bit) {
    RadixBufs b;
    b.passes = (end_bit + kRadixBits - 1) / kRadixBits;
    b.nparts = (count + kPartKeys - 1) / kPartKeys;
    b.ka = ar.take<uint32_t>(count);
    b.kb = ar.take<uint32_t>(count);
    b.va = ar.take<int32_t>(count);
    b.vb = ar.take<int32_t>(count);
    const size_t before = (ar.used + 255) & ~size_t(255);
    b.hist = ar.take<unsigned>((size_t)kMaxPasses * kRadix);
    b.tickets = ar.take<unsigned>(kMaxPasses);
    b.lookback = ar.take<uint32_t>((size_t)b.passes * b.nparts * kRadix);
    b.zero_bytes = ar.used - before;
    return b;
}

// Zeroes a sort's histogram, tickets and look-back words (before a producer
// that fills the histogram, see KeyHist).
static int radix_clear(const RadixBufs &b, cudaStream_t s) {
    if (cudaMemsetAsync(b.hist, 0, b.zero_bytes, s) != cudaSuccess)
        return check_launch("sort workspace memset");
    return SPLAT_OK;
}

static KeyHist key_hist(const RadixBufs &b, int end_bit) {
    return KeyHist{b.hist, b.passes, end_bit};
}

// Sorts (ka, va) by the low end_bit bits of the keys.  Returns the buffers
// holding the result; the last pass writes the values to vals_final instead
// when it is given.  hist_ready: radix_clear ran and the producer of the keys
// filled the histogram (KeyHist), so neither the clearing nor the histogram
// pass runs here.
static int radix_sort(uint32_t *status, uint32_t spin, const RadixBufs &b, Count count,
                      int end_bit, int32_t *vals_final, const uint32_t **keys_sorted,
                      const int32_t **vals_sorted, cudaStream_t s, bool hist_ready = false) {
    if (count.cap > (long long)kLbMask)
        return fail(SPLAT_ERR_OVERFLOW, "sort of %lld keys exceeds %u", count.cap, kLbMask);
    *keys_sorted = b.ka;
    *vals_sorted = b.va;
    if (count.cap == 0) return SPLAT_OK;
    if (!hist_ready) {
        if (int rc = radix_clear(b, s)) return rc;
        HistArgs h{b.ka, count, b.passes, end_bit, b.hist};
        long long blocks = (count.cap + 256 * 16 - 1) / (256 * 16);
        if (blocks > 152 * 8) blocks = 152 * 8;
        if (blocks < 1) blocks = 1;
        radix_hist_kernel<<<(unsigned)blocks, 256, 0, s>>>(h);
        if (int rc = check_launch("radix_hist_kernel")) return rc;
    }
    uint32_t *kin = b.ka, *kout = b.kb;
    int32_t *vin = b.va, *vout = b.vb;
    for (int d = 0; d < b.passes; ++d) {
        const bool last = d == b.passes - 1;
        PassArgs pa;
        pa.keys_in = kin;
        pa.vals_in = vin;
        pa.keys_out = kout;
        pa.vals_out = (last && vals_final) ? vals_final : vout;
        pa.count = count;
        pa.shift = d * kRadixBits;
        pa.mask = (1u << min(kRadixBits, end_bit - d * kRadixBits)) - 1u;
        pa.hist = b.hist + d * kRadix;
        pa.lookback = b.lookback + (size_t)d * b.nparts * kRadix;
        pa.ticket = b.tickets + d;
        pa.status = status;
        pa.spin_limit = spin;
        onesweep_kernel<<<(unsigned)b.nparts, kSortThreads, 0, s>>>(pa);
        if (int rc = check_launch("onesweep_kernel")) return rc;
        kin = kout;
        kout = (kin == b.ka) ? b.kb : b.ka;
        int32_t *vw = pa.vals_out;
        vin = vw;
        vout = (vw == b.va) ? b.vb : b.va;
    }
    *keys_sorted = kin;
    *vals_sorted = vin;
    return SPLAT_OK;
}

// ---------------------------------------------------------------------------
// Stage 1 input: 32-bit depth keys (Gaussians that hit no tile sort last).

// Grid-stride, with the depth sort's digit counts (KeyHist).
__global__ void __launch_bounds__(256) depth_keys_kernel(int n, const float *depths,
                                                         const int32_t *radii, uint32_t *keys,
                                                         int32_t *vals, KeyHist h) {
    __shared__ unsigned sh[kMaxPasses][kRadix];
    key_hist_zero(sh);
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = radii[i] > 0 ? __float_as_uint(depths[i]) : 0xffffffffu;
        keys[i] = k;
        vals[i] = i;
        key_hist_add(h, sh, k);
    }
    __syncthreads();
    key_hist_flush(h, sh);
}

// Blocks of the depth-key pass: about 4 keys per thread, at most 8 per SM.
static unsigned depth_key_blocks(long long n) {
    return (unsigned)std::max(1ll, std::min(152ll * 8, (n + 256 * 4 - 1) / (256 * 4)));
}

// ---------------------------------------------------------------------------
// Stage 2: emission in depth order, in two kernels.
//
// emit_offsets_kernel: each Gaussian's first slot, an exclusive scan of the
// tile counts in depth order.  Large partitions (4096 positions per block of
// 1024 threads) keep the look-back chain short: the decoupled look-back's
// inclusive prefixes advance by one window of partitions per L2 round trip,
// so its latency grows with the number of partitions.
// emit_expand_kernel: a block owns 256 consecutive positions of the depth
// order; their tile rectangles are expanded cooperatively so that
// consecutive threads write consecutive slots.  No waiting on other blocks.

// The tile grid an entry is emitted into: one grid (single view), or the
// grid of the entry's view, whose tiles are numbered from its tile_base
// (batched views).
struct SingleGrid {
    unsigned tiles_x, tiles_y, bw;
    __device__ __forceinline__ void of(int, unsigned &tx_n, unsigned &ty_n, unsigned &base) const {
        tx_n = tiles_x;
        ty_n = tiles_y;
        base = 0;
    }
};

struct ViewGrid {
    const splat_view *views;
    int nviews;
    unsigned bw;
    __device__ __forceinline__ void of(int entry, unsigned &tx_n, unsigned &ty_n,
                                       unsigned &base) const {
        const splat_view &v = views[view_by_entry(views, nviews, (uint32_t)entry)];
        tx_n = v.tiles_x;
        ty_n = v.tiles_y;
        base = v.tile_base;
    }
};

constexpr int kEmitBlock = 256;
constexpr int kOffThreads = 1024;
constexpr int kOffItems = 4;
constexpr int kOffPart = kOffThreads * kOffItems;

template <class Grid>
struct EmitOffsetsArgs {
    int n;
    const int32_t *order;  // Gaussian ids in depth order
    const float *xys;
    const int32_t *radii;
    Grid grid;
    int32_t *offs;              // [n] first slot of each depth position (saturated at INT32_MAX)
    unsigned long long *words;  // [0] ticket, [1 + b] look-back word of block b
    uint32_t *status;
    uint32_t spin_limit;
};

template <class Grid>
__device__ __forceinline__ int rect_count(const EmitOffsetsArgs<Grid> &a, int g) {
    if (g < 0 || g >= a.n) return 0;
    const int rad = a.radii[g];
    if (rad <= 0) return 0;
    unsigned tx_n, ty_n, base;
    a.grid.of(g, tx_n, ty_n, base);
    const float2 c = make_float2(a.xys[2 * (size_t)g], a.xys[2 * (size_t)g + 1]);
    const TileRect r = tile_rect(c, (float)rad, tx_n, ty_n, a.grid.bw);
    return (int)((r.x1 - r.x0) * (r.y1 - r.y0));
}

template <class Grid>
__global__ void __launch_bounds__(kOffThreads) emit_offsets_kernel(EmitOffsetsArgs<Grid> a) {
    __shared__ unsigned long long s_warp[kOffThreads / 32];
    __shared__ unsigned long long s_base;
    __shared__ int s_part;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_part = (int)atomicAdd(&a.words[0], 1ull);
    __syncthreads();
    const int part = s_part;
    const long long first = (long long)part * kOffPart + (long long)t * kOffItems;
    int cnt[kOffItems];
    long long run = 0;
#pragma unroll
    for (int k = 0; k < kOffItems; ++k) {
        const long long pos = first + k;
        cnt[k] = pos < a.n ? rect_count(a, a.order[pos]) : 0;
        run += cnt[k];
    }
    // block exclusive scan of the per-thread totals
    unsigned long long v = (unsigned long long)run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kOffThreads / 32 ? s_warp[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        if (lane < kOffThreads / 32) s_warp[lane] = w;  // inclusive over warps
        const unsigned long long block_total = __shfl_sync(0xffffffffu, w, kOffThreads / 32 - 1);
        unsigned long long *words = a.words + 1;
        unsigned long long excl = 0;
        if (part == 0) {
            if (lane == 0) publish(&words[0], kFlagPrefix | (block_total & kValueMask));
        } else {
            if (lane == 0) publish(&words[part], kFlagAggregate | (block_total & kValueMask));
            excl = warp_lookback(words, part, a.spin_limit, a.status);
            if (lane == 0) publish(&words[part], kFlagPrefix | ((excl + block_total) & kValueMask));
        }
        if (lane == 0) s_base = excl;
    }
    __syncthreads();
    unsigned long long o = s_base + (warp ? s_warp[warp - 1] : 0ull) + (v - (unsigned long long)run);
#pragma unroll
    for (int k = 0; k < kOffItems; ++k) {
        const long long pos = first + k;
        if (pos < a.n) a.offs[pos] = o < 0x7fffffffull ? (int32_t)o : 0x7fffffff;
        o += (unsigned long long)cnt[k];
    }
}

template <class Grid>
struct EmitExpandArgs {
    int n;
    const int32_t *order;
    const int32_t *offs;
    const float *xys;
    const int32_t *radii;
    Grid grid;
    Count count;
    uint32_t *tile_out;
    int32_t *id_out;
    uint32_t *status;
    KeyHist hist;  // the tile sort's digit counts of the written keys
};

template <class Grid>
__global__ void __launch_bounds__(kEmitBlock) emit_expand_kernel(EmitExpandArgs<Grid> a) {
    __shared__ unsigned s_hist[kMaxPasses][kRadix];
    __shared__ int s_off[kEmitBlock];
    __shared__ int4 s_info[kEmitBlock];  // (first tile, tiles per row of the grid, width, id)
    __shared__ float s_rw[kEmitBlock];   // 1 / width
    __shared__ int s_total;
    const int t = threadIdx.x;
    const int k0 = blockIdx.x * kEmitBlock;
    const int k = k0 + t;
    const int last = min(a.n, k0 + kEmitBlock) - 1;
    const int base = a.offs[k0];
    key_hist_zero(s_hist);
    int cnt = 0;
    if (k < a.n) {
        const int g = a.order[k];
        if (g >= 0 && g < a.n) {
            const int rad = a.radii[g];
            if (rad > 0) {
                unsigned tx_n, ty_n, tbase;
                a.grid.of(g, tx_n, ty_n, tbase);
                const float2 c = make_float2(a.xys[2 * (size_t)g], a.xys[2 * (size_t)g + 1]);
                const TileRect r = tile_rect(c, (float)rad, tx_n, ty_n, a.grid.bw);
                s_info[t] = make_int4((int)(tbase + r.y0 * tx_n + r.x0), (int)tx_n,
                                      (int)(r.x1 - r.x0), g);
                s_rw[t] = 1.f / (float)(r.x1 - r.x0);
                cnt = (int)((r.x1 - r.x0) * (r.y1 - r.y0));
            }
        } else {
            raise_status(a.status, DEV_BAD_ID);
        }
        // offsets relative to the block's first slot; a saturated offset
        // (past any capacity) lands past the count and is reported below
        s_off[t] = (int)min((long long)a.offs[k] - base, 0x3fffffffll);
        if (k == last) s_total = (int)min((long long)a.offs[k] - base + cnt, 0x3fffffffll);
    } else {
        s_off[t] = 0x7fffffff;  // never an owner
    }
    __syncthreads();
    const int total = s_total;
    const long long count = a.count.get();
    if (blockIdx.x == 0 && t == 0 && a.count.dev && *a.count.dev > a.count.cap)
        raise_status(a.status, DEV_CAPACITY);
    // slots past the count are not written (and reported once)
    const int lim = (int)max(0ll, min((long long)total, count - (long long)base));
    if (t == 0 && lim < total) raise_status(a.status, DEV_EMIT_OVERFLOW);
    for (int s = t; s < lim; s += kEmitBlock) {
        // owner: last j with s_off[j] <= s (skips Gaussians with no slots);
        // s_off[0] = 0 <= s, so a fixed-depth search over 256 entries
        int j = 0;
#pragma unroll
        for (int step = kEmitBlock / 2; step > 0; step >>= 1)
            if (s_off[j + step] <= s) j += step;
        const int kk = s - s_off[j];
        const int4 info = s_info[j];
        const int w = info.z;
        // kk / w through the float reciprocal, corrected to the exact
        // quotient: the quotient is a row of the rectangle (below 2^16), so
        // the estimate's relative error of ~2^-22 puts it off by at most one
        int qy = (int)((float)kk * s_rw[j]);
        int rx = kk - qy * w;
        if (rx < 0) { --qy; rx += w; }
        if (rx >= w) { ++qy; rx -= w; }
        const int slot = base + s;
        const uint32_t key = (uint32_t)(info.x + qy * info.y + rx);
        a.tile_out[slot] = key;
        a.id_out[slot] = info.w;
        key_hist_add(a.hist, s_hist, key);
    }
    __syncthreads();
    key_hist_flush(a.hist, s_hist);
}

// ---------------------------------------------------------------------------
// Optional outputs with the reference's intermediate layouts: the unsorted
// emission in Gaussian order (forward.cu:135-179) and the sorted 64-bit keys.

struct EmitRefArgs {
    int n;
    const float *xys, *depths;
    const int32_t *radii, *cum;
    unsigned tiles_x, tiles_y, bw;
    Count count;
    unsigned long long *keys;
    int32_t *ids;
    uint32_t *status;
};

__global__ void __launch_bounds__(kEmitBlock) emit_ref_kernel(EmitRefArgs a) {
    __shared__ int s_off[kEmitBlock + 1];
    __shared__ int s_start[kEmitBlock];
    __shared__ unsigned s_x0[kEmitBlock], s_y0[kEmitBlock], s_w[kEmitBlock];
    __shared__ int s_dbits[kEmitBlock];
    __shared__ int s_warp[kEmitBlock / 32];
    const int t = threadIdx.x;
    const int g = blockIdx.x * kEmitBlock + t;
    int cnt = 0;
    if (g < a.n) {
        const int rad = a.radii[g];
        if (rad > 0) {
            const float2 c = make_float2(a.xys[2 * (size_t)g], a.xys[2 * (size_t)g + 1]);
            const TileRect r = tile_rect(c, (float)rad, a.tiles_x, a.tiles_y, a.bw);
            s_x0[t] = r.x0;
            s_y0[t] = r.y0;
            s_w[t] = r.x1 - r.x0;
            cnt = (int)((r.x1 - r.x0) * (r.y1 - r.y0));
            s_dbits[t] = __float_as_int(a.depths[g]);
        }
        s_start[t] = g == 0 ? 0 : a.cum[g - 1];
    }
    const int lane = t & 31, warp = t >> 5;
    int v = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
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
    const long long count = a.count.get();
    for (int s = t; s < total; s += kEmitBlock) {
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
        if (slot < 0 || slot >= count) {
            raise_status(a.status, DEV_EMIT_OVERFLOW);
            continue;
        }
        const unsigned long long tile = (unsigned long long)(ty * a.tiles_x + tx);
        a.keys[slot] = (tile << 32) | (unsigned long long)(long long)s_dbits[j];
        a.ids[slot] = blockIdx.x * kEmitBlock + j;
    }
}

__global__ void compose_keys_kernel(Count count, const uint32_t *tiles, const int32_t *ids,
                                    const float *depths, int n, unsigned long long *keys) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count.get()) return;
    const int g = ids[i];
    const int dbits = (g >= 0 && g < n) ? __float_as_int(depths[g]) : 0;
    keys[i] = ((unsigned long long)tiles[i] << 32) | (unsigned long long)(long long)dbits;
}

// ---------------------------------------------------------------------------
// Tile bin edges by search over the sorted tile ids.  Writes every tile,
// (0, 0) when empty, so no zeroing pass is needed (the reference memsets then
// marks the boundaries, forward.cu:184-208).


// One warp per tile: lanes 0-15 find the first key >= t, lanes 16-31 the
// first key >= t + 1, each half by a 16-way search (16 probes per step, a
// ballot picks the interval), so a tile costs ~6 dependent loads instead of
// the ~2 log2(I) of a binary search.  Invariant: the answer lies in [lo, hi].
__global__ void __launch_bounds__(256) tile_bins_kernel(const uint32_t *keys, Count cnt,
                                                        int ntiles, int2 *bins) {
    const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
    const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= ntiles) return;  // whole warps
    const uint32_t x = (uint32_t)t + (uint32_t)half;
    long long lo = 0, hi = cnt.get();
    for (;;) {
        const bool active = hi - lo > 16;
        if (!__any_sync(0xffffffffu, active)) break;
        const long long step = (hi - lo + 15) >> 4;
        const long long idx = lo + hl * step;
        const bool ge = !active || idx >= hi || keys[idx] >= x;
        const unsigned b = (__ballot_sync(0xffffffffu, ge) >> (half * 16)) & 0xffffu;
        if (active) {
            if (b == 0) {
                lo += 15 * step + 1;  // every probe < x
            } else {
                const int f = __ffs(b) - 1;
                if (f == 0) {
                    hi = lo;  // keys[lo] >= x
                } else {
                    const long long p = lo + f * step;
                    lo += (f - 1) * step + 1;
                    hi = min(hi, p);
                }
            }
        }
    }
    const long long idx = lo + hl;
    const bool ge = idx >= hi || keys[idx] >= x;
    const unsigned b = (__ballot_sync(0xffffffffu, ge) >> (half * 16)) & 0xffffu;
    const long long first = b ? lo + (__ffs(b) - 1) : hi;
    const long long next = __shfl_sync(0xffffffffu, first, 16);
    if (lane == 0) bins[t] = first < next ? make_int2((int)first, (int)next) : make_int2(0, 0);
}

// ---------------------------------------------------------------------------
// Host side.

static int bit_length(unsigned v) {
    int b = 0;
    while ((v >> b) != 0) ++b;
    return b;
}

struct SortLayout {
    RadixBufs g;                 // Gaussians by depth
    unsigned long long *words;   // emission look-back words
    int32_t *offs;               // first slot of each depth position
    RadixBufs s;                 // intersections by tile
};

static SortLayout sort_layout(Arena &ar, const splat_params &p, long long count) {
    SortLayout L;
    const long long n = p.num_points;
    L.g = radix_layout(ar, n, 32);
    L.words = ar.take<unsigned long long>((size_t)((n + kOffPart - 1) / kOffPart + 1));
    L.offs = ar.take<int32_t>((size_t)n);
    const int tile_bits = std::max(1, bit_length(n_tiles(p) - 1));
    L.s = radix_layout(ar, count, tile_bits);
    return L;
}

size_t sort_workspace_bytes(const splat_params &p, long long count) {
    Arena ar{nullptr, 0};
    sort_layout(ar, p, count);
    return ar.used + 256;
}

int launch_sort_and_bin(const splat_params &p, Count count, const float *xys,
                        const float *depths, const int32_t *radii, const int32_t *cum,
                        int32_t *ids_sorted, int2 *bins, long long *isect_out,
                        int32_t *ids_unsorted_out, long long *keys_sorted_out, void *ws,
                        size_t ws_bytes, cudaStream_t s) {
    const unsigned tx = tiles_x(p), ty = tiles_y(p), T = tx * ty;
    const int n = (int)p.num_points;
    Arena ar{static_cast<char *>(ws), ws_bytes};
    const SortLayout L = sort_layout(ar, p, count.cap);
    if (!ar.fits())
        return fail(SPLAT_ERR_WORKSPACE, "sort workspace too small: need %zu bytes, got %zu",
                    ar.used, ws_bytes);
    if (count.cap == 0 || n == 0) {
        if (cudaMemsetAsync(bins, 0, sizeof(int2) * T, s) != cudaSuccess)
            return check_launch("tile_bins memset");
        return SPLAT_OK;
    }
    // reference-layout intermediates, on request only
    if (isect_out || ids_unsorted_out) {
        if (!isect_out || !ids_unsorted_out)
            return fail(SPLAT_ERR_INVALID_ARG, "isect_ids and gaussian_ids are requested together");
        EmitRefArgs e;
        e.n = n;
        e.xys = xys; e.depths = depths; e.radii = radii; e.cum = cum;
        e.tiles_x = tx; e.tiles_y = ty; e.bw = p.block_width;
        e.count = count;
        e.keys = reinterpret_cast<unsigned long long *>(isect_out);
        e.ids = ids_unsorted_out;
        e.status = p.device_status;
        emit_ref_kernel<<<(n + kEmitBlock - 1) / kEmitBlock, kEmitBlock, 0, s>>>(e);
        if (int rc = check_launch("emit_ref_kernel")) return rc;
    }
    // 1. Gaussians by depth
    if (int rc = radix_clear(L.g, s)) return rc;
    depth_keys_kernel<<<depth_key_blocks(n), 256, 0, s>>>(n, depths, radii, L.g.ka, L.g.va,
                                                          key_hist(L.g, 32));
    if (int rc = check_launch("depth_keys_kernel")) return rc;
    const uint32_t *gkeys;
    const int32_t *order;
    const Count all{nullptr, n, n};
    if (int rc = radix_sort(p.device_status, spin_limit(p), L.g, all, 32, nullptr, &gkeys, &order, s,
                            true))
        return rc;
    // 2. emission in depth order
    const int oblocks = (n + kOffPart - 1) / kOffPart;
    if (cudaMemsetAsync(L.words, 0, sizeof(unsigned long long) * (size_t)(oblocks + 1), s) != cudaSuccess)
        return check_launch("emission workspace memset");
    const SingleGrid grid{tx, ty, p.block_width};
    EmitOffsetsArgs<SingleGrid> eo;
    eo.n = n;
    eo.order = order;
    eo.xys = xys;
    eo.radii = radii;
    eo.grid = grid;
    eo.offs = L.offs;
    eo.words = L.words;
    eo.status = p.device_status;
    eo.spin_limit = spin_limit(p);
    emit_offsets_kernel<<<oblocks, kOffThreads, 0, s>>>(eo);
    if (int rc = check_launch("emit_offsets_kernel")) return rc;
    EmitExpandArgs<SingleGrid> e;
    e.n = n;
    e.order = order;
    e.offs = L.offs;
    e.xys = xys;
    e.radii = radii;
    e.grid = grid;
    e.count = count;
    e.tile_out = L.s.ka;
    e.id_out = L.s.va;
    e.status = p.device_status;
    const int tile_bits = std::max(1, bit_length(T - 1));
    e.hist = key_hist(L.s, tile_bits);
    if (int rc = radix_clear(L.s, s)) return rc;
    emit_expand_kernel<<<(n + kEmitBlock - 1) / kEmitBlock, kEmitBlock, 0, s>>>(e);
    if (int rc = check_launch("emit_expand_kernel")) return rc;
    // 3. stable sort by tile id
    const uint32_t *tiles_sorted;
    const int32_t *ids_final;
    if (int rc = radix_sort(p.device_status, spin_limit(p), L.s, count, tile_bits, ids_sorted,
                            &tiles_sorted, &ids_final, s, true))
        return rc;
    if (keys_sorted_out) {
        compose_keys_kernel<<<(unsigned)((count.cap + 255) / 256), 256, 0, s>>>(
            count, tiles_sorted, ids_sorted, depths, n,
            reinterpret_cast<unsigned long long *>(keys_sorted_out));
        if (int rc = check_launch("compose_keys_kernel")) return rc;
    }
    // 4. bins
    tile_bins_kernel<<<(unsigned)(((long long)T * 32 + 255) / 256), 256, 0, s>>>(tiles_sorted, count,
                                                                           (int)T, bins);
    return check_launch("tile_bins_kernel");
}

// ---------------------------------------------------------------------------
// Batched views: the same pipeline over all entries of all views, tiles
// numbered view after view, plus the rasterizers' work order.

constexpr int kCostBits = 24;
constexpr uint32_t kCostMask = (1u << kCostBits) - 1u;

// Ascending keys put the longest tile lists first (lists longer than 2^24
// share the first key).
__global__ void tile_cost_kernel(const int2 *bins, int ntiles, uint32_t *keys, int32_t *vals) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    const int2 r = bins[t];
    const unsigned cost = (unsigned)max(0, r.y - r.x);
    keys[t] = kCostMask - min(cost, kCostMask);
    vals[t] = t;
}

struct BatchSortLayout {
    RadixBufs g;                // entries by depth
    unsigned long long *words;  // emission look-back words
    int32_t *offs;              // first slot of each depth position
    RadixBufs s;                // intersections by tile
    RadixBufs o;                // tiles by list length
};

static BatchSortLayout batch_sort_layout(Arena &ar, const splat_batch &b, long long count) {
    BatchSortLayout L;
    const long long e = (long long)b.num_entries, T = (long long)b.num_tiles;
    L.g = radix_layout(ar, e, 32);
    L.words = ar.take<unsigned long long>((size_t)((e + kOffPart - 1) / kOffPart + 1));
    L.offs = ar.take<int32_t>((size_t)e);
    L.s = radix_layout(ar, count, std::max(1, bit_length((unsigned)(T - 1))));
    L.o = radix_layout(ar, T, kCostBits);
    return L;
}

size_t batch_sort_workspace_bytes(const splat_batch &b, long long count) {
    Arena ar{nullptr, 0};
    batch_sort_layout(ar, b, count);
    return ar.used + 256;
}

int launch_batch_sort_and_bin(const splat_batch &b, Count count, const float *xys,
                              const float *depths, const int32_t *radii, int32_t *ids_sorted,
                              int2 *bins, int32_t *order, void *ws, size_t ws_bytes,
                              cudaStream_t s) {
    const int e = (int)b.num_entries, T = (int)b.num_tiles;
    Arena ar{static_cast<char *>(ws), ws_bytes};
    const BatchSortLayout L = batch_sort_layout(ar, b, count.cap);
    if (!ar.fits())
        return fail(SPLAT_ERR_WORKSPACE, "batch sort workspace too small: need %zu bytes, got %zu",
                    ar.used, ws_bytes);
    const uint32_t spin = spin_limit(b);
    if (count.cap > 0 && e > 0) {
        // 1. entries by depth
        if (int rc = radix_clear(L.g, s)) return rc;
        depth_keys_kernel<<<depth_key_blocks(e), 256, 0, s>>>(e, depths, radii, L.g.ka, L.g.va,
                                                              key_hist(L.g, 32));
        if (int rc = check_launch("depth_keys_kernel")) return rc;
        const uint32_t *gkeys;
        const int32_t *order_d;
        const Count all{nullptr, e, e};
        if (int rc = radix_sort(b.device_status, spin, L.g, all, 32, nullptr, &gkeys, &order_d, s,
                                true))
            return rc;
        // 2. emission in depth order, each entry into its view's tiles
        const int oblocks = (e + kOffPart - 1) / kOffPart;
        if (cudaMemsetAsync(L.words, 0, sizeof(unsigned long long) * (size_t)(oblocks + 1), s) !=
            cudaSuccess)
            return check_launch("emission workspace memset");
        const ViewGrid grid{b.views, (int)b.num_views, b.block_width};
        EmitOffsetsArgs<ViewGrid> eo;
        eo.n = e;
        eo.order = order_d;
        eo.xys = xys;
        eo.radii = radii;
        eo.grid = grid;
        eo.offs = L.offs;
        eo.words = L.words;
        eo.status = b.device_status;
        eo.spin_limit = spin;
        emit_offsets_kernel<<<oblocks, kOffThreads, 0, s>>>(eo);
        if (int rc = check_launch("emit_offsets_kernel")) return rc;
        EmitExpandArgs<ViewGrid> ex;
        ex.n = e;
        ex.order = order_d;
        ex.offs = L.offs;
        ex.xys = xys;
        ex.radii = radii;
        ex.grid = grid;
        ex.count = count;
        ex.tile_out = L.s.ka;
        ex.id_out = L.s.va;
        ex.status = b.device_status;
        const int tile_bits = std::max(1, bit_length((unsigned)(T - 1)));
        ex.hist = key_hist(L.s, tile_bits);
        if (int rc = radix_clear(L.s, s)) return rc;
        emit_expand_kernel<<<(e + kEmitBlock - 1) / kEmitBlock, kEmitBlock, 0, s>>>(ex);
        if (int rc = check_launch("emit_expand_kernel")) return rc;
        // 3. stable sort by global tile id; 4. bins
        const uint32_t *tiles_sorted;
        const int32_t *ids_final;
        if (int rc = radix_sort(b.device_status, spin, L.s, count, tile_bits, ids_sorted,
                                &tiles_sorted, &ids_final, s, true))
            return rc;
        tile_bins_kernel<<<(unsigned)(((long long)T * 32 + 255) / 256), 256, 0, s>>>(
            tiles_sorted, count, (int)T, bins);
        if (int rc = check_launch("tile_bins_kernel")) return rc;
    } else if (cudaMemsetAsync(bins, 0, sizeof(int2) * (size_t)T, s) != cudaSuccess) {
        return check_launch("tile_bins memset");
    }
    // 5. work order: longest list first
    tile_cost_kernel<<<(T + 255) / 256, 256, 0, s>>>(bins, T, L.o.ka, L.o.va);
    if (int rc = check_launch("tile_cost_kernel")) return rc;
    const uint32_t *ck;
    const int32_t *cv;
    const Count tiles{nullptr, T, T};
    return radix_sort(b.device_status, spin, L.o, tiles, kCostBits, order, &ck, &cv, s);
}

}  // namespace splat
