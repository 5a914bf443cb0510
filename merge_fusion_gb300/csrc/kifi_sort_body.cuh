// kifi_sort_body.cuh -- the device bodies of the onesweep radix sort
// (kifi_sort.cu): digit histograms, the pass set-up and one digit pass.
// Their shared memory is passed in, so that a kernel running several stages
// (the batched fusion queue, kifi_integrate.cu) can overlay it.
#pragma once

#include "kifi_api_util.h"

namespace kifi {
namespace sort_detail {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kKeysPerThread = 8;
constexpr int kTile = kThreads * kKeysPerThread;  // 2048
constexpr int kRadix = 256;
constexpr unsigned long long kSpinLimit = 1ull << 22;
constexpr int kLookAhead = 8;  // predecessor look-back words fetched per round

constexpr unsigned long long kFlagAggregate = 1ull << 30;
constexpr unsigned long long kFlagInclusive = 2ull << 30;
constexpr unsigned long long kCountMask = (1ull << 30) - 1;

__device__ __forceinline__ void sort_prepare_body(const SortScratch& s, int passes) {
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) s.hist[i] = 0u;
    if (threadIdx.x < passes) s.tile_counter[threadIdx.x] = s.first_tile;
    if (threadIdx.x == 0) *s.epoch += 1ull;
}

// all `passes` digit histograms in one read of the keys
struct SortHistSmem {
    unsigned int h[kSortMaxPasses][kRadix];
};
template <typename K>
__device__ __forceinline__ void sort_histogram_body(const K* __restrict__ keys, const unsigned int* __restrict__ n_ptr,
                                                    const SortScratch& s, int passes, unsigned int blk,
                                                    unsigned int nblk, SortHistSmem& sm) {
    auto& h = sm.h;
    for (int i = threadIdx.x; i < passes * kRadix; i += kThreads) (&h[0][0])[i] = 0u;
    __syncthreads();
    const size_t n = min((size_t)*n_ptr, s.max_n);
    for (size_t i = (size_t)blk * kThreads + threadIdx.x; i < n;
         i += (size_t)nblk * kThreads) {
        const K k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(unsigned int)(k >> (8 * p)) & 0xffu], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += kThreads) {
        unsigned int c = (&h[0][0])[i];
        if (c) atomicAdd(&s.hist[i], c);
    }
}

__device__ __forceinline__ unsigned int lanemask_lt() {
    unsigned int m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_volatile_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// One digit pass of kBits bits (radix R = 2^kBits, R / kThreads digits per
// thread in the scans and the look-back: one for 8-bit digits, four for the
// frame keys' 10-bit digits).
template <int kBits>
struct SortPassSmem {
    unsigned int warp_hist[kWarps][(1 << kBits) + 1];  // last column: out-of-range keys
    unsigned int digit_base[1 << kBits];
    unsigned int pass_offset[1 << kBits];
    unsigned int wsum[kWarps];
    unsigned int tile_id;
};
template <bool kWithValues, typename K, int kBits>
__device__ __forceinline__ void sort_pass_body(const K* __restrict__ keys_in, K* __restrict__ keys_out,
                                               const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ vals_out,
                                               const unsigned int* __restrict__ n_ptr, const SortScratch& s,
                                               int pass, unsigned int blk, SortPassSmem<kBits>& sm) {
    constexpr int R = 1 << kBits;
    constexpr int D = R / kThreads;
    constexpr int kLA = D == 1 ? kLookAhead : kLookAhead / 2;  // look-back words per digit and round
    static_assert(D >= 1 && D * kThreads == R, "whole digits per thread");
    auto& warp_hist = sm.warp_hist;
    auto& digit_base = sm.digit_base;
    auto& pass_offset = sm.pass_offset;
    auto& wsum = sm.wsum;
    auto& tile_id = sm.tile_id;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned int n = (unsigned int)min((size_t)*n_ptr, s.max_n);
    const unsigned int n_tiles = (n + kTile - 1) / kTile;
    // Grids are sized before the key count exists.  CTAs beyond the tile
    // count leave before the tile counter: n_tiles CTAs (or the whole grid,
    // when smaller) take every tile, and the counter sees only them.
    if (blk >= n_tiles) return;
    const int shift = pass * kBits;
    const unsigned long long gen = (*s.epoch & 0xffffffffull) << 32;
    unsigned long long* lb = s.lookback + (size_t)pass * s.max_tiles * R;

    bool have_offsets = false;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) tile_id = atomicAdd(&s.tile_counter[pass], 1u);
        __syncthreads();
        const unsigned int tile = tile_id;
        if (tile >= n_tiles) break;  // (CTAs without a tile leave before any other work)
        for (int i = threadIdx.x; i < kWarps * (R + 1); i += kThreads) (&warp_hist[0][0])[i] = 0u;
        if (!have_offsets) {
            // exclusive scan of this pass's global digit histogram: thread t
            // holds digits t*D .. t*D + D - 1
            unsigned int c[D], sum = 0;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                c[q] = s.hist[pass * R + threadIdx.x * D + q];
                sum += c[q];
            }
            unsigned int x = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) wsum[warp] = x;
            __syncthreads();
            unsigned int run = x - sum;
            for (int w = 0; w < warp; ++w) run += wsum[w];
#pragma unroll
            for (int q = 0; q < D; ++q) {
                pass_offset[threadIdx.x * D + q] = run;
                run += c[q];
            }
            have_offsets = true;  // read after the next barrier, before the scatter
        }
        __syncthreads();  // warp_hist cleared

        const unsigned int base = tile * kTile + warp * (32 * kKeysPerThread);
        K k[kKeysPerThread];
        uint32_t v[kKeysPerThread];
        unsigned int rank[kKeysPerThread];
        int dig[kKeysPerThread];
#pragma unroll
        for (int j = 0; j < kKeysPerThread; ++j) {
            unsigned int i = base + j * 32 + lane;
            bool ok = i < n;
            k[j] = ok ? keys_in[i] : (K)0;
            if (kWithValues) v[j] = ok ? vals_in[i] : 0u;
            dig[j] = ok ? (int)((unsigned int)(k[j] >> shift) & (unsigned int)(R - 1)) : R;
        }
        // stable warp-local ranks: lanes with equal digits, in (j, lane) order
#pragma unroll
        for (int j = 0; j < kKeysPerThread; ++j) {
            unsigned int peers = __match_any_sync(0xffffffffu, dig[j]);
            unsigned int before = warp_hist[warp][dig[j]];
            rank[j] = before + __popc(peers & lanemask_lt());
            __syncwarp();
            if (lane == __ffs(peers) - 1) warp_hist[warp][dig[j]] = before + __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        // per digit d = threadIdx.x + q * kThreads: counts across warps ->
        // exclusive prefix over warps
        unsigned int tile_count[D];
#pragma unroll
        for (int q = 0; q < D; ++q) {
            const int d = threadIdx.x + q * kThreads;
            unsigned int tc = 0;
            for (int w = 0; w < kWarps; ++w) {
                unsigned int c = warp_hist[w][d];
                warp_hist[w][d] = tc;
                tc += c;
            }
            tile_count[q] = tc;
        }
        // decoupled look-back for the thread's digits
        if (tile == 0) {
#pragma unroll
            for (int q = 0; q < D; ++q) {
                const int d = threadIdx.x + q * kThreads;
                st_volatile_u64(lb + d, gen | kFlagInclusive | tile_count[q]);
                digit_base[d] = pass_offset[d];
            }
        } else {
#pragma unroll
            for (int q = 0; q < D; ++q)
                st_volatile_u64(lb + (size_t)tile * R + threadIdx.x + q * kThreads,
                                gen | kFlagAggregate | tile_count[q]);
            // Walk back kLA predecessor words per digit and round: the loads of
            // a round are independent, so a chain of aggregate-only tiles
            // costs one memory latency per kLA tiles, not one per tile.
            unsigned int excl[D];
            int t[D];
            unsigned int pending = 0;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                excl[q] = 0;
                t[q] = (int)tile - 1;
                pending |= 1u << q;
            }
            unsigned long long spins = 0;
            while (pending) {
                unsigned long long w[D][kLA];
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    const int d = threadIdx.x + q * kThreads;
#pragma unroll
                    for (int i = 0; i < kLA; ++i)
                        w[q][i] = ((pending >> q) & 1u) && t[q] - i >= 0
                                      ? ld_volatile_u64(lb + (size_t)(t[q] - i) * R + d)
                                      : 0ull;
                }
                // consume each digit's words in order, up to the first inclusive
                // one or the first one not yet published
                bool stalled_any = false;
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    if (!((pending >> q) & 1u)) continue;
                    int used = 0;
                    bool done = false, stalled = false;
#pragma unroll
                    for (int i = 0; i < kLA; ++i) {
                        if (done || stalled || t[q] - i < 0) continue;
                        const unsigned long long x = w[q][i];
                        if ((x & 0xffffffff00000000ull) != gen || (x & (3ull << 30)) == 0) {
                            stalled = true;
                            continue;
                        }
                        excl[q] += (unsigned int)(x & kCountMask);
                        ++used;
                        done = (x & kFlagInclusive) != 0;
                    }
                    t[q] -= used;
                    if (done || t[q] < 0) pending &= ~(1u << q);
                    else if (stalled) stalled_any = true;
                }
                if (stalled_any && ++spins > s.spin_limit) {
                    atomicOr(s.status, KIFI_DEV_ERR_TIMEOUT);
                    break;
                }
            }
#pragma unroll
            for (int q = 0; q < D; ++q) {
                const int d = threadIdx.x + q * kThreads;
                st_volatile_u64(lb + (size_t)tile * R + d, gen | kFlagInclusive | ((excl[q] + tile_count[q]) & kCountMask));
                digit_base[d] = pass_offset[d] + excl[q];
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kKeysPerThread; ++j) {
            if (dig[j] == R) continue;
            unsigned int pos = digit_base[dig[j]] + warp_hist[warp][dig[j]] + rank[j];
            if (pos >= n) {  // only reachable after a timed-out look-back
                atomicOr(s.status, KIFI_DEV_ERR_TIMEOUT);
                continue;
            }
            keys_out[pos] = k[j];
            if (kWithValues) vals_out[pos] = v[j];
        }
    }
}

}  // namespace sort_detail
}  // namespace kifi
