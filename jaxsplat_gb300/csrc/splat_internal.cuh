// splat_internal.cuh -- shared host/device plumbing of libsplat.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda/atomic>
#include <cuda_runtime.h>

#include "../../include/splat.h"

namespace splat {

// Bits of the device status word (splat_params::device_status).  Kernels
// OR them in instead of trapping, so a failed check never takes the context
// down; the host reads the word at its next synchronisation point.
enum : uint32_t {
    DEV_LOOKBACK_TIMEOUT = 1u << 0,  // a decoupled look-back wait ran out
    DEV_EMIT_OVERFLOW = 1u << 1,     // an intersection slot fell outside [0, count)
    DEV_SORT_OVERFLOW = 1u << 2,     // a radix scatter position fell outside [0, count)
    DEV_SCAN_OVERFLOW = 1u << 3,     // intersection total does not fit int32
    DEV_BAD_TILE = 1u << 4,          // a sorted key named a tile outside the grid
    DEV_BAD_ID = 1u << 5,            // a sorted list entry named a Gaussian outside [0, N)
    DEV_CAPACITY = 1u << 6,          // the device-side count exceeded the buffers' capacity
};

// An intersection count known either on the host or in device memory (the
// int64 total the projection writes), clamped to the buffers' capacity.
struct Count {
    const long long *dev;  // null: use `host`
    long long host;
    long long cap;
    __device__ __forceinline__ long long get() const {
        const long long v = dev ? *dev : host;
        return v < 0 ? 0 : (v < cap ? v : cap);
    }
};

constexpr uint32_t kDefaultSpinLimit = 1u << 22;

// Batched views: the view that owns an entry, a tile or a pixel.  Views are
// laid out in order, so every base field is non-decreasing over the table and
// the owner is the last view whose base is <= the key.
template <class Key, class Field>
__device__ __forceinline__ int view_search(const splat_view *v, int n, Key key, Field field) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (field(v[mid]) <= key) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int view_by_entry(const splat_view *v, int n, uint32_t entry) {
    return view_search(v, n, entry, [](const splat_view &x) { return x.entry_base; });
}
__device__ __forceinline__ int view_by_tile(const splat_view *v, int n, uint32_t tile) {
    return view_search(v, n, tile, [](const splat_view &x) { return x.tile_base; });
}
__device__ __forceinline__ int view_by_pixel(const splat_view *v, int n, uint64_t pix) {
    return view_search(v, n, pix, [](const splat_view &x) { return x.pixel_base; });
}

__device__ __forceinline__ void raise_status(uint32_t *status, uint32_t bits) {
    if (status) atomicOr(status, bits);
}

// Look-back words: two flag bits over a 62-bit value.  The value travels
// inside the word and nothing else is read on its strength, so relaxed
// device-scope loads and stores are enough.
constexpr unsigned long long kFlagAggregate = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kValueMask = (1ull << 62) - 1ull;

__device__ __forceinline__ void publish(unsigned long long *slot, unsigned long long word) {
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> a(*slot);
    a.store(word, cuda::memory_order_relaxed);
}

// Poll `slot` until it holds a flagged word.  Gives up after `limit` polls
// (with a short sleep between polls after the first few), raises
// DEV_LOOKBACK_TIMEOUT and returns a prefix-flagged zero so callers finish.
__device__ __forceinline__ unsigned long long wait_flagged(unsigned long long *slot,
                                                           uint32_t limit, uint32_t *status) {
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> a(*slot);
    for (uint32_t i = 0; i < limit; ++i) {
        const unsigned long long w = a.load(cuda::memory_order_relaxed);
        if (w & (kFlagAggregate | kFlagPrefix)) return w;
        if (i > 32) __nanosleep(64);
    }
    raise_status(status, DEV_LOOKBACK_TIMEOUT);
    return kFlagPrefix;
}

// Warp-parallel decoupled look-back (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016).  Called by all 32
// lanes of one warp on behalf of partition `part` (> 0); returns the
// exclusive prefix of partition `part` in every lane.
__device__ __forceinline__ unsigned long long warp_lookback(unsigned long long *words, int part,
                                                            uint32_t limit, uint32_t *status) {
    const int lane = threadIdx.x & 31;
    unsigned long long excl = 0;
    int base = part - 1;
    while (true) {
        const int j = base - lane;
        unsigned long long w = kFlagPrefix;  // lanes past partition 0 contribute nothing
        if (j >= 0) w = wait_flagged(&words[j], limit, status);
        const unsigned prefix_lanes = __ballot_sync(0xffffffffu, (w & kFlagPrefix) != 0);
        // lanes up to and including the nearest prefix-flagged one contribute
        const int stop = prefix_lanes ? __ffs(prefix_lanes) - 1 : 31;
        unsigned long long v = (lane <= stop && j >= 0) ? (w & kValueMask) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (prefix_lanes) return excl;
        base -= 32;
    }
}

// Host-side helpers -----------------------------------------------------------

struct Arena {
    // Bump allocator over a caller-provided workspace (256-byte aligned
    // sub-allocations).  With base == nullptr it only measures.
    char *base;
    size_t cap;
    size_t used = 0;
    template <typename T>
    T *take(size_t count) {
        used = (used + 255) & ~size_t(255);
        T *p = base ? reinterpret_cast<T *>(base + used) : nullptr;
        used += count * sizeof(T);
        return p;
    }
    bool fits() const { return used <= cap; }
};

inline unsigned tiles_x(const splat_params &p) { return (p.img_width + p.block_width - 1) / p.block_width; }
inline unsigned tiles_y(const splat_params &p) { return (p.img_height + p.block_width - 1) / p.block_width; }
inline unsigned n_tiles(const splat_params &p) { return tiles_x(p) * tiles_y(p); }

inline uint32_t spin_limit(const splat_params &p) {
    return p.spin_limit ? p.spin_limit : kDefaultSpinLimit;
}
inline uint32_t spin_limit(const splat_batch &b) {
    return b.spin_limit ? b.spin_limit : kDefaultSpinLimit;
}

// Sets the thread-local error message and returns `code`.
int fail(int code, const char *fmt, ...);
int check_launch(const char *what);

}  // namespace splat
