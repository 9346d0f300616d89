// k_scan.cuh -- device-wide exclusive prefix sum (u32) and stable LSD radix
// sort of (key, u32 value) pairs for u32 and u64 keys.
//
// Every pipeline count -> offset step (pair counts per body, rows per slot
// group and per body, CSR incidences per body, colour histograms) is a
// k_scan_partials + k_scan_apply pair of launches (tile sums, then each tile
// scanned with the lower tiles' sums; one k_scan_excl launch, a single-pass
// look-back scan, for a single tile); every sort (LBVH Morton keys of worlds
// with scenes beyond the shared-memory trees, the dynamic-body work order,
// warm-start row keys, incidence lists) is one k_radix_hist launch plus one
// k_radix_pass launch per 8-bit digit, each pass with decoupled look-back.
// All of them open with griddepcontrol.wait and so chain with programmatic
// dependent launch.
//
// Look-back protocol (k_radix_pass, k_scan_excl).  The input is cut into tiles; CTA b takes tiles b,
// b + grid, b + 2 grid, ... in order, and the grid is at most what the SMs
// hold at once, so the lowest unfinished tile always belongs to a running
// CTA that is working on it: every wait ends.  A tile publishes its
// aggregate, then walks back over lower tiles, adding aggregates until it
// meets an inclusive prefix, and publishes its own inclusive prefix.  Status
// words are (value << 32) | (epoch << 2) | flag.  The epoch is the high half
// of a 64-bit control word whose low half counts the CTAs of the launch that
// are done: each CTA reads the epoch first and counts itself last, and the
// last one advances the epoch for the next launch.  Words left by an earlier
// launch so carry an older epoch and read as "not ready", and the status
// array is never cleared.  Launches that share one control word and status
// array must not overlap, which the stream order (with griddepcontrol.wait
// first in every kernel) guarantees.  Each wait is also bounded: after
// kLookbackPolls polls the CTA raises kErrTimeout, takes the missing value
// as 0 and finishes; scatter addresses stay bounds-checked, so a timed-out
// launch writes wrong values in range and the host reports DIO_ERR_TIMEOUT.
#pragma once

#include <algorithm>
#include <cstdint>

#include "engine.cuh"

namespace dio {

constexpr uint32_t kLbAggregate = 1u, kLbInclusive = 2u;
constexpr uint32_t kLookbackPolls = 1u << 22;

struct Lookback {
    unsigned long long* ctl;     // (epoch << 32) | CTAs of the launch done
    unsigned long long* status;  // per tile (256 digit columns in the radix passes)
    uint32_t* err;               // error flag word
};

__device__ __forceinline__ unsigned long long lb_load(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void lb_store(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t lb_tag(uint32_t epoch) { return (epoch & 0x3FFFFFFFu) << 2; }
__device__ __forceinline__ unsigned long long lb_word(uint32_t value, uint32_t epoch, uint32_t flag) {
    return ((unsigned long long)value << 32) | (lb_tag(epoch) | flag);
}

// the launch's epoch; one thread per CTA, before the CTA touches a status word
__device__ __forceinline__ uint32_t lb_epoch(const unsigned long long* ctl) { return (uint32_t)(lb_load(ctl) >> 32); }
// one thread per CTA, after the CTA's last status access
__device__ __forceinline__ void lb_done(unsigned long long* ctl) {
    const unsigned long long old = atomicAdd(ctl, 1ull);
    if ((uint32_t)old == gridDim.x - 1u) atomicExch(ctl, (old & ~0xFFFFFFFFull) + (1ull << 32));
}

// Exclusive prefix of `tile` in status column `col` (row stride `stride`),
// one thread reading kLbWindow lower tiles at a time (independent loads, so
// a run of aggregates costs one round trip per window, not per tile).
constexpr int kLbWindow = 8;
__device__ __forceinline__ uint32_t lb_walk(const Lookback& lb, uint32_t tile, uint32_t col, uint32_t stride,
                                            uint32_t epoch) {
    const uint32_t tag = lb_tag(epoch);
    const unsigned long long before_first = lb_word(0u, epoch, kLbInclusive);
    uint32_t prefix = 0, polls = 0;
    int64_t p = (int64_t)tile - 1;
    bool done = false;
    while (!done && p >= 0) {
        unsigned long long s[kLbWindow];
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k)
            s[k] = p - k >= 0 ? lb_load(lb.status + (size_t)(p - k) * stride + col) : before_first;
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k) {
            if (done) continue;
            unsigned long long x = s[k];
            while (((uint32_t)x & ~3u) != tag || ((uint32_t)x & 3u) == 0u) {
                if (++polls > kLookbackPolls) {
                    atomicOr(lb.err, kErrTimeout);
                    x = before_first;
                    break;
                }
                x = lb_load(lb.status + (size_t)(p - k) * stride + col);
            }
            prefix += (uint32_t)(x >> 32);
            done = ((uint32_t)x & 3u) == kLbInclusive;
        }
        p -= kLbWindow;
    }
    return prefix;
}

// The same for a one-column status array, one warp reading 32 x K lower
// tiles per window (lane l the K tiles at distances l K + 1 .. l K + K);
// all 32 lanes call it and get the prefix.
template <int K = 1>
__device__ __forceinline__ uint32_t lb_walk_warp(const Lookback& lb, uint32_t tile, uint32_t epoch, uint32_t lane) {
    const uint32_t tag = lb_tag(epoch);
    uint32_t prefix = 0;
    int64_t p = (int64_t)tile - 1;  // nearest tile of this window
    while (p >= 0) {
        uint32_t v[K], f[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int64_t q = p - (int64_t)(lane * K + k);
            v[k] = 0u;
            f[k] = kLbInclusive;  // before tile 0: an inclusive 0
            if (q >= 0) {
                const unsigned long long s = lb_load(lb.status + q);
                v[k] = (uint32_t)(s >> 32);
                f[k] = ((uint32_t)s & ~3u) == tag ? ((uint32_t)s & 3u) : 0u;
            }
        }
        // wait for the entries not yet published, then sum up to this lane's
        // first inclusive entry
        uint32_t part = 0, first = K;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int64_t q = p - (int64_t)(lane * K + k);
            if (first < (uint32_t)K) continue;  // beyond this lane's inclusive entry
            for (uint32_t polls = 0; f[k] == 0u; ++polls) {
                if (polls >= kLookbackPolls) {
                    atomicOr(lb.err, kErrTimeout);
                    v[k] = 0u;
                    f[k] = kLbInclusive;
                    break;
                }
                const unsigned long long s = lb_load(lb.status + q);
                v[k] = (uint32_t)(s >> 32);
                f[k] = ((uint32_t)s & ~3u) == tag ? ((uint32_t)s & 3u) : 0u;
            }
            part += v[k];
            if (f[k] == kLbInclusive) first = (uint32_t)k;
        }
        const uint32_t incl = __ballot_sync(0xFFFFFFFFu, first < (uint32_t)K);
        const uint32_t upto = incl ? (uint32_t)(__ffs(incl) - 1) : 31u;
        uint32_t x = lane <= upto ? part : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
        prefix += x;
        if (incl) break;
        p -= 32 * K;
    }
    return prefix;
}

// Exclusive prefix of each thread's v over the launch: tiles in order, then
// threads in order within a tile.  Every thread of the CTA calls it once per
// tile (the CTA's tiles in increasing order); *tile_end receives the
// inclusive prefix at the tile's end (the launch total after the last
// tile).  s_warp holds THREADS / 32 words, s_pair 2; ep is the launch's
// epoch (lb_epoch, stored before the first call and read after its barrier).
template <int THREADS, int K = 1>
__device__ __forceinline__ uint32_t tile_exclusive(uint32_t v, uint32_t tile, const uint32_t* s_ep, const Lookback& lb,
                                                   uint32_t* s_warp, uint32_t* s_pair, uint32_t* tile_end) {
    constexpr int NW = THREADS / 32;
    static_assert(NW <= 32, "one warp scans the warp totals");
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;  // inclusive over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31u) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const uint32_t ep = *s_ep;
        const uint32_t wv = lane < (uint32_t)NW ? s_warp[lane] : 0u;
        uint32_t wi = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= (uint32_t)o) wi += y;
        }
        if (lane < (uint32_t)NW) s_warp[lane] = wi - wv;
        const uint32_t agg = __shfl_sync(0xFFFFFFFFu, wi, 31);
        unsigned long long* slot = lb.status + tile;
        uint32_t pre = 0u;
        if (tile == 0u) {
            if (lane == 0u) lb_store(slot, lb_word(agg, ep, kLbInclusive));
        } else {
            if (lane == 0u) lb_store(slot, lb_word(agg, ep, kLbAggregate));
            pre = lb_walk_warp<K>(lb, tile, ep, lane);
            if (lane == 0u) lb_store(slot, lb_word(pre + agg, ep, kLbInclusive));
        }
        if (lane == 0u) {
            s_pair[0] = pre;
            s_pair[1] = pre + agg;
        }
    }
    __syncthreads();
    const uint32_t r = s_pair[0] + s_warp[warp] + (x - v);
    *tile_end = s_pair[1];
    __syncthreads();  // s_warp and s_pair serve the next tile
    return r;
}

// ---- exclusive prefix sum ---------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanTile = (uint32_t)(kScanThreads * kScanItems);

// out[i] = in[0] + ... + in[i-1] for i < m (in and out may alias), where
// m = n, or min(*n_dev, n) when the live count is on the device; total
// (optional) receives in[0] + ... + in[m-1]
static __global__ void __launch_bounds__(kScanThreads)
    k_scan_excl(const uint32_t* in, uint32_t* out, uint32_t n, const uint32_t* n_dev, uint32_t* total, Lookback lb) {
    pdl_enter();
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_ep, s_pair[2];
    if (threadIdx.x == 0) s_ep = lb_epoch(lb.ctl);
    if (n_dev) n = min(*n_dev, n);
    if (n == 0u && total && blockIdx.x == 0 && threadIdx.x == 0) *total = 0u;
    const bool in16 = (reinterpret_cast<uintptr_t>(in) & 15u) == 0u;
    const bool out16 = (reinterpret_cast<uintptr_t>(out) & 15u) == 0u;
    const uint32_t tiles = (uint32_t)(((size_t)n + kScanTile - 1) / kScanTile);
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const size_t base = (size_t)tile * kScanTile + (size_t)threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
        const bool full = base + kScanItems <= n;
        if (full && in16) {
            const uint4* s4 = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
            for (int k = 0; k < kScanItems / 4; ++k) {
                const uint4 q = s4[k];
                v[4 * k + 0] = q.x;
                v[4 * k + 1] = q.y;
                v[4 * k + 2] = q.z;
                v[4 * k + 3] = q.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < kScanItems; ++j) v[j] = base + j < n ? in[base + j] : 0u;
        }
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) sum += v[j];
        uint32_t end = 0;
        uint32_t run = tile_exclusive<kScanThreads>(sum, tile, &s_ep, lb, s_warp, s_pair, &end);
        if (total && tile + 1u == tiles && threadIdx.x == 0) *total = end;
        if (full && out16) {
            uint4* d4 = reinterpret_cast<uint4*>(out + base);
#pragma unroll
            for (int k = 0; k < kScanItems / 4; ++k) {
                uint4 q;
                q.x = run;
                run += v[4 * k + 0];
                q.y = run;
                run += v[4 * k + 1];
                q.z = run;
                run += v[4 * k + 2];
                q.w = run;
                run += v[4 * k + 3];
                d4[k] = q;
            }
        } else {
#pragma unroll
            for (int j = 0; j < kScanItems; ++j) {
                if (base + j < n) out[base + j] = run;
                run += v[j];
            }
        }
    }
    if (threadIdx.x == 0) lb_done(lb.ctl);
}

// The same prefix sum as two launches without waits: k_scan_partials sums
// each tile, k_scan_apply adds the partials of the lower tiles (one load a
// thread) and scans its tile.  With programmatic dependent launch the
// second launch overlaps the first's tail; neither waits on another CTA.
__device__ __forceinline__ void scan_load_tile(const uint32_t* in, uint32_t n, size_t base, bool in16,
                                               uint32_t v[kScanItems]) {
    if (base + kScanItems <= n && in16) {
        const uint4* s4 = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            const uint4 q = s4[k];
            v[4 * k + 0] = q.x;
            v[4 * k + 1] = q.y;
            v[4 * k + 2] = q.z;
            v[4 * k + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) v[j] = base + j < n ? in[base + j] : 0u;
    }
}
__device__ __forceinline__ uint32_t block_sum_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    // exclusive over the CTA's threads; *total = the CTA's sum
    constexpr int NW = kScanThreads / 32;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31u) s_warp[warp] = x;
    __syncthreads();
    uint32_t wofs = 0, all = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        const uint32_t sw = s_warp[w];
        wofs += (uint32_t)w < warp ? sw : 0u;
        all += sw;
    }
    __syncthreads();
    *total = all;
    return wofs + x - v;
}
static __global__ void __launch_bounds__(kScanThreads)
    k_scan_partials(const uint32_t* in, uint32_t n, const uint32_t* n_dev, uint32_t* partials) {
    pdl_enter();
    __shared__ uint32_t s_warp[kScanThreads / 32];
    if (n_dev) n = min(*n_dev, n);
    const bool in16 = (reinterpret_cast<uintptr_t>(in) & 15u) == 0u;
    const uint32_t tiles = (uint32_t)(((size_t)n + kScanTile - 1) / kScanTile);
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        uint32_t v[kScanItems];
        scan_load_tile(in, n, (size_t)tile * kScanTile + (size_t)threadIdx.x * kScanItems, in16, v);
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) sum += v[j];
        uint32_t all = 0;
        block_sum_scan(sum, s_warp, &all);
        if (threadIdx.x == 0) partials[tile] = all;
    }
}
static __global__ void __launch_bounds__(kScanThreads)
    k_scan_apply(const uint32_t* in, uint32_t* out, uint32_t n, const uint32_t* n_dev, const uint32_t* partials,
                 uint32_t* total) {
    pdl_enter();
    __shared__ uint32_t s_warp[kScanThreads / 32];
    if (n_dev) n = min(*n_dev, n);
    if (n == 0u && total && blockIdx.x == 0 && threadIdx.x == 0) *total = 0u;
    const bool in16 = (reinterpret_cast<uintptr_t>(in) & 15u) == 0u;
    const bool out16 = (reinterpret_cast<uintptr_t>(out) & 15u) == 0u;
    const uint32_t tiles = (uint32_t)(((size_t)n + kScanTile - 1) / kScanTile);
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const size_t base = (size_t)tile * kScanTile + (size_t)threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
        scan_load_tile(in, n, base, in16, v);
        // partials of the lower tiles, one or more a thread
        uint32_t low = 0;
        for (uint32_t t = threadIdx.x; t < tile; t += kScanThreads) low += partials[t];
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) sum += v[j];
        // one pass: the tile's own thread sums and the lower partials
        uint32_t lowall = 0, tileall = 0;
        block_sum_scan(low, s_warp, &lowall);
        uint32_t run = lowall + block_sum_scan(sum, s_warp, &tileall);
        if (total && tile + 1u == tiles && threadIdx.x == 0) *total = lowall + tileall;
        if (base + kScanItems <= n && out16) {
            uint4* d4 = reinterpret_cast<uint4*>(out + base);
#pragma unroll
            for (int k = 0; k < kScanItems / 4; ++k) {
                uint4 q;
                q.x = run;
                run += v[4 * k + 0];
                q.y = run;
                run += v[4 * k + 1];
                q.z = run;
                run += v[4 * k + 2];
                q.w = run;
                run += v[4 * k + 3];
                d4[k] = q;
            }
        } else {
#pragma unroll
            for (int j = 0; j < kScanItems; ++j) {
                if (base + j < n) out[base + j] = run;
                run += v[j];
            }
        }
    }
}

// ---- LSD radix sort ---------------------------------------------------
constexpr int kRadixThreads = 256;  // one thread per digit value
constexpr int kRadixHistThreads = 256;
constexpr int kRadixMaxPasses = 8;
template <class K>
__host__ __device__ constexpr int radix_items() {
    return sizeof(K) == 8 ? 8 : 16;
}
template <class K>
__host__ __device__ constexpr uint32_t radix_tile() {
    return (uint32_t)(kRadixThreads * radix_items<K>());
}
template <class K>
__host__ __device__ constexpr size_t radix_smem_bytes() {  // the tile's keys and values in digit order
    return (size_t)radix_tile<K>() * (sizeof(K) + 4);
}

template <class K>
__device__ __forceinline__ uint32_t radix_digit(K key, uint32_t shift, uint32_t mask) {
    return (uint32_t)(key >> shift) & mask;
}

// Lanes of the warp whose digit (width bits, < 256) equals this lane's
// (warp-level multi-split: one ballot per digit bit); 0 for lanes whose
// d is >= 256 (no key)
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, uint32_t width) {
    uint32_t peers = __ballot_sync(0xFFFFFFFFu, d < 256u);
    for (uint32_t b = 0; b < width; ++b) {
        const uint32_t bit = (d >> b) & 1u;
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, bit);
        peers &= bit ? bal : ~bal;
    }
    return d < 256u ? peers : 0u;
}

// Digit counts of every pass in one read of the keys, then (in the CTA that
// finishes last) their exclusive sums: bases[p * 256 + d] = keys whose
// digit p is below d.  hist is zero at rest and left zero.  A warp whose
// 32 keys share a digit (the high digits of near-sorted keys) adds 32 once.
template <class K>
__global__ void __launch_bounds__(kRadixHistThreads)
    k_radix_hist(const K* __restrict__ keys, uint32_t n, uint32_t begin_bit, uint32_t end_bit, uint32_t* hist,
                 uint32_t* done, uint32_t* bases) {
    pdl_enter();
    __shared__ uint32_t sh[kRadixMaxPasses * 256];
    __shared__ bool s_last;
    const uint32_t passes = (end_bit - begin_bit + 7u) / 8u;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t i = threadIdx.x; i < passes * 256u; i += blockDim.x) sh[i] = 0u;
    __syncthreads();
    // warp-uniform trip count: every lane takes part in the votes
    const size_t wstride = (size_t)gridDim.x * blockDim.x;
    for (size_t i0 = (size_t)blockIdx.x * blockDim.x + (size_t)warp * 32u; i0 < n; i0 += wstride) {
        const size_t i = i0 + lane;
        const bool ok = i < n;
        const bool whole = __all_sync(0xFFFFFFFFu, ok);
        const K k = ok ? keys[i] : K(0);
        for (uint32_t p = 0; p < passes; ++p) {
            const uint32_t shift = begin_bit + 8u * p;
            const uint32_t width = min(8u, end_bit - shift);
            const uint32_t d = radix_digit(k, shift, (1u << width) - 1u);
            if (whole && __all_sync(0xFFFFFFFFu, d == __shfl_sync(0xFFFFFFFFu, d, 0))) {
                if (lane == 0u) atomicAdd(&sh[p * 256u + d], 32u);
            } else if (ok) {
                atomicAdd(&sh[p * 256u + d], 1u);
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * 256u; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // one warp per pass: 8 digits a lane, then a warp scan
    for (uint32_t p = warp; p < passes; p += blockDim.x / 32u) {
        uint32_t c[8], s = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            c[k] = __ldcg(&hist[p * 256u + lane * 8u + k]);
            s += c[k];
        }
        uint32_t x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        uint32_t run = x - s;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            bases[p * 256u + lane * 8u + k] = run;
            run += c[k];
            hist[p * 256u + lane * 8u + k] = 0u;
        }
    }
    if (threadIdx.x == 0) *done = 0u;
}

// One stable counting pass on digit (key >> shift) & (2^width - 1).  A tile
// holds radix_tile<K>() keys, warp w its w-th slice, lane-minor.  A key's
// place in the tile's digit order is (keys of smaller digits in the tile) +
// (keys of its digit in lower warps) + (earlier in its warp, by ballot peer
// ranks); the keys are staged in that order in shared memory and written
// out so that consecutive threads write consecutive places of one digit.
// Thread d owns digit d: its tile count, the look-back on status column d,
// and the global place of the digit's first key in this tile: bases[d] +
// (keys of digit d in lower tiles).
template <class K>
__global__ void __launch_bounds__(kRadixThreads)
    k_radix_pass(const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
                 uint32_t* __restrict__ vout, uint32_t n, uint32_t shift, uint32_t width,
                 const uint32_t* __restrict__ bases, Lookback lb) {
    pdl_enter();
    constexpr int IT = radix_items<K>();
    constexpr int NW = kRadixThreads / 32;
    constexpr uint32_t TILE = radix_tile<K>();
    extern __shared__ __align__(16) unsigned char radix_smem[];
    K* s_k = reinterpret_cast<K*>(radix_smem);
    uint32_t* s_v = reinterpret_cast<uint32_t*>(s_k + TILE);
    __shared__ uint32_t s_cnt[NW][256];
    __shared__ uint32_t s_tdig[256];  // tile place of each digit's first key
    __shared__ uint32_t s_goff[256];  // global place minus tile place, per digit
    __shared__ uint32_t s_wsum[NW];
    __shared__ uint32_t s_ep;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_ep = lb_epoch(lb.ctl);
    const uint32_t mask = (1u << width) - 1u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t tiles = (uint32_t)(((size_t)n + TILE - 1) / TILE);
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
#pragma unroll
        for (int w = 0; w < NW; ++w) s_cnt[w][tid] = 0u;
        __syncthreads();
        const size_t wbase = (size_t)tile * TILE + (size_t)warp * (IT * 32);
        K key[IT];
        uint32_t val[IT], dig[IT], rank[IT];
#pragma unroll
        for (int j = 0; j < IT; ++j) {
            const size_t idx = wbase + (size_t)j * 32u + lane;
            const bool ok = idx < n;
            key[j] = ok ? kin[idx] : K(0);
            val[j] = ok ? vin[idx] : 0u;
            dig[j] = ok ? radix_digit(key[j], shift, mask) : 256u;
        }
#pragma unroll
        for (int j = 0; j < IT; ++j) {
            const uint32_t d = dig[j];
            const uint32_t peers = digit_peers(d, width);
            const uint32_t before = peers ? s_cnt[warp][d] : 0u;
            rank[j] = before + __popc(peers & lt);
            __syncwarp();
            if (peers && (peers & lt) == 0u) s_cnt[warp][d] = before + __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        // thread tid = digit d: warp offsets, tile count, tile place
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            const uint32_t c = s_cnt[w][tid];
            s_cnt[w][tid] = cnt;
            cnt += c;
        }
        uint32_t x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31u) s_wsum[warp] = x;
        __syncthreads();
        uint32_t wofs = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) wofs += (uint32_t)w < warp ? s_wsum[w] : 0u;
        const uint32_t tdig = wofs + x - cnt;
        s_tdig[tid] = tdig;
        const uint32_t ep = s_ep;
        unsigned long long* slot = lb.status + (size_t)tile * 256u + tid;
        uint32_t pre = 0u;
        if (tile == 0u) {
            lb_store(slot, lb_word(cnt, ep, kLbInclusive));
        } else {
            lb_store(slot, lb_word(cnt, ep, kLbAggregate));
            pre = lb_walk(lb, tile, tid, 256u, ep);
            lb_store(slot, lb_word(pre + cnt, ep, kLbInclusive));
        }
        s_goff[tid] = bases[tid] + pre - tdig;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < IT; ++j) {
            const uint32_t d = dig[j];
            if (d < 256u) {
                const uint32_t place = s_tdig[d] + s_cnt[warp][d] + rank[j];
                s_k[place] = key[j];
                s_v[place] = val[j];
            }
        }
        __syncthreads();
        const size_t rest = (size_t)n - (size_t)tile * TILE;
        const uint32_t tile_n = rest < TILE ? (uint32_t)rest : TILE;
        for (uint32_t i = tid; i < tile_n; i += kRadixThreads) {
            const K k = s_k[i];
            const uint32_t g = s_goff[radix_digit(k, shift, mask)] + i;
            if (g < n) {
                kout[g] = k;
                vout[g] = s_v[i];
            }
        }
        __syncthreads();  // the shared arrays serve the next tile
    }
    if (tid == 0) lb_done(lb.ctl);
}

// ---- host side ----------------------------------------------------------
// Buffers of the scan and sort kernels for one stream: the look-back control
// word and status array, the digit histograms, and the sort's ping-pong
// arrays.  Launches through one ScanSort must be stream-ordered.
struct ScanSort {
    unsigned long long* ctl = nullptr;
    unsigned long long* status = nullptr;
    uint32_t* hist = nullptr;   // kRadixMaxPasses * 256, zero at rest
    uint32_t* done = nullptr;   // CTAs of k_radix_hist finished, zero at rest
    uint32_t* bases = nullptr;  // kRadixMaxPasses * 256
    uint32_t* partials = nullptr;  // per-tile sums of the two-launch scan
    void* kalt = nullptr;       // max_sort keys of 8 bytes
    uint32_t* valt = nullptr;   // max_sort values
    uint32_t* err = nullptr;    // not owned
    uint32_t max_sort = 0, max_scan = 0;
    int sms = 1;
    // CTAs that the SMs hold at once: the grid limit of the look-back kernels
    int scan_ctas = 1, pass_ctas32 = 1, pass_ctas64 = 1;
    uint64_t launches = 0;        // kernels launched through this object
    uint64_t* counter = nullptr;  // optional: the owner's launch counter, advanced too
    void counted(uint64_t k) {
        launches += k;
        if (counter) *counter += k;
    }

    // status words for sorts of max_sort keys, scans of max_scan entries and
    // other look-back launches of up to max_tiles tiles
    static size_t status_words(uint32_t max_sort, uint32_t max_scan, size_t max_tiles) {
        const size_t radix_tiles = ((size_t)max_sort + radix_tile<unsigned long long>() - 1) /
                                   radix_tile<unsigned long long>();
        const size_t scan_tiles = ((size_t)max_scan + kScanTile - 1) / kScanTile;
        return std::max<size_t>(1, std::max(std::max(radix_tiles * 256u, scan_tiles), max_tiles));
    }
    size_t max_status = 0;  // status words allocated
    cudaError_t init(uint32_t max_sort_n, uint32_t max_scan_n, uint32_t* err_flags, cudaStream_t s,
                     size_t max_tiles = 0) {
        max_sort = max_sort_n;
        max_scan = max_scan_n;
        err = err_flags;
        int dev = 0, per = 0;
        cudaError_t e;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_scan_excl, kScanThreads, 0)) != cudaSuccess)
            return e;
        scan_ctas = std::max(1, per) * sms;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_radix_pass<uint32_t>, kRadixThreads,
                                                               radix_smem_bytes<uint32_t>())) != cudaSuccess)
            return e;
        pass_ctas32 = std::max(1, per) * sms;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_radix_pass<unsigned long long>, kRadixThreads,
                                                               radix_smem_bytes<unsigned long long>())) !=
            cudaSuccess)
            return e;
        pass_ctas64 = std::max(1, per) * sms;
        const size_t sw = status_words(max_sort, max_scan, max_tiles);
        max_status = sw;
        if ((e = cudaMalloc(&ctl, 8)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&status, sw * 8)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&hist, kRadixMaxPasses * 256 * 4)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&done, 4)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&bases, kRadixMaxPasses * 256 * 4)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&partials, (((size_t)max_scan + kScanTile - 1) / kScanTile + 1) * 4)) != cudaSuccess)
            return e;
        if ((e = cudaMalloc(&kalt, std::max<size_t>(1, max_sort) * 8)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&valt, std::max<size_t>(1, max_sort) * 4)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(ctl, 0, 8, s)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(status, 0, sw * 8, s)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(hist, 0, kRadixMaxPasses * 256 * 4, s)) != cudaSuccess) return e;
        return cudaMemsetAsync(done, 0, 4, s);
    }
    void release() {
        for (void* p : {(void*)ctl, (void*)status, (void*)hist, (void*)done, (void*)bases, (void*)partials, kalt,
                        (void*)valt})
            if (p) cudaFree(p);
        ctl = status = nullptr;
        hist = done = bases = partials = valt = nullptr;
        kalt = nullptr;
    }
    Lookback lookback() const { return Lookback{ctl, status, err}; }

    // exclusive sum of n entries (n <= max_scan), or of the first *n_dev of
    // them; total (optional) receives the sum
    cudaError_t scan(const uint32_t* in, uint32_t* out, uint32_t n, bool pdl, cudaStream_t s,
                     const uint32_t* n_dev = nullptr, uint32_t* total = nullptr) {
        if (n > max_scan) return cudaErrorInvalidValue;
        if (n == 0 && !total) return cudaSuccess;
        const int g = (int)std::max<size_t>(1, ((size_t)n + kScanTile - 1) / kScanTile);
        if (g == 1) {  // one tile: the single launch (its look-back has nothing to wait for)
            counted(1);
            return launch_k(pdl, k_scan_excl, 1, kScanThreads, 0, s, in, out, n, n_dev, total, lookback());
        }
        counted(2);
        cudaError_t e = launch_k(pdl, k_scan_partials, g, kScanThreads, 0, s, in, n, n_dev, partials);
        if (e != cudaSuccess) return e;
        return launch_k(true, k_scan_apply, g, kScanThreads, 0, s, in, out, n, n_dev, (const uint32_t*)partials,
                        total);
    }

    // stable sort of n pairs by key bits [begin_bit, end_bit) (n <= max_sort);
    // kin/vin are left as they were
    template <class K>
    cudaError_t sort_pairs(const K* kin, K* kout, const uint32_t* vin, uint32_t* vout, uint32_t n, uint32_t begin_bit,
                           uint32_t end_bit, bool pdl, cudaStream_t s) {
        if (n == 0) return cudaSuccess;
        if (n > max_sort || end_bit > 8 * sizeof(K) || begin_bit > end_bit) return cudaErrorInvalidValue;
        cudaError_t e;
        if (end_bit == begin_bit) {
            if ((e = cudaMemcpyAsync(kout, kin, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                return e;
            return cudaMemcpyAsync(vout, vin, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
        }
        const uint32_t passes = (end_bit - begin_bit + 7u) / 8u;
        const int gh = std::max(1, std::min((int)((n + 4095u) / 4096u), 2 * sms));
        if ((e = launch_k(pdl, k_radix_hist<K>, gh, kRadixHistThreads, 0, s, kin, n, begin_bit, end_bit, hist, done,
                          bases)) != cudaSuccess)
            return e;
        const int cap = sizeof(K) == 8 ? pass_ctas64 : pass_ctas32;
        const int g = (int)std::min<size_t>(((size_t)n + radix_tile<K>() - 1) / radix_tile<K>(), (size_t)cap);
        const K* ks = kin;
        const uint32_t* vs = vin;
        for (uint32_t p = 0; p < passes; ++p) {
            // the last pass lands in (kout, vout)
            const bool to_out = ((passes - 1u - p) & 1u) == 0u;
            K* kd = to_out ? kout : reinterpret_cast<K*>(kalt);
            uint32_t* vd = to_out ? vout : valt;
            const uint32_t shift = begin_bit + 8u * p;
            const uint32_t width = std::min(8u, end_bit - shift);
            if ((e = launch_k(true, k_radix_pass<K>, g, kRadixThreads, radix_smem_bytes<K>(), s, ks, vs, kd, vd, n,
                              shift, width, (const uint32_t*)(bases + 256u * p), lookback())) != cudaSuccess)
                return e;
            ks = kd;
            vs = vd;
        }
        counted(1 + passes);
        return cudaSuccess;
    }
};

}  // namespace dio
