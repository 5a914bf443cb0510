// kifi_sort.cu -- stable LSD radix sort of 32-bit keys (optionally carrying
// 32-bit values) on sm_103a, the GPU counterpart of kifi::util::radix_sort
// (KinectFission/kifi/util/algorithm.h:63-134: four stable 8-bit passes,
// each an exclusive scan of 256 digit counts, numeric.h:78-108).
//
// The key count is read from device memory, so a sort can be enqueued
// behind the kernel that produces the keys without a host round trip and
// captured in a CUDA graph.
//
// A frame's 30-bit new keys take three 10-bit digit passes instead: the
// frame's set-up kernel prepares them and the splat counts their digits
// (kifi_integrate.cu), so that sort is three launches of k_sort_pass_frame.
//
// Structure (one "onesweep" kernel per digit pass):
//  * k_sort_prepare: zero the digit histograms and the dynamic tile
//    counters, bump the look-back generation tag.
//  * k_sort_histogram: one read of the keys builds all four 256-bin digit
//    histograms (shared-memory counters, then one global atomic per bin).
//  * k_sort_pass: persistent CTAs take 2048-key tiles in increasing order
//    from an atomic counter.  Each warp ranks its keys with
//    __match_any_sync (a stable rank among lanes holding the same digit),
//    per-warp digit counts are scanned across warps in shared memory, the
//    tile's counts are published to a decoupled look-back array and the
//    tile's global offsets are resolved by walking back over predecessor
//    tiles.  Keys (and values) are scattered to their final position of the
//    pass.
// The look-back words pack {generation:32 | status:2 | count:30}, so the
// count and its flag are one atomic 64-bit store and stale words of an
// earlier sort are ignored without clearing.  Every wait on a predecessor is
// bounded: after kSpinLimit polls (or the limit a test sets) the kernel
// raises KIFI_DEV_ERR_TIMEOUT in the caller's status word and carries on with
// what it has -- every store stays inside the output buffers -- so a broken
// invariant can never hang the GPU.
#include <atomic>

#include "kifi_api_util.h"

namespace kifi {
namespace {

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

__global__ void k_sort_prepare(SortScratch s, int passes) { sort_prepare_body(s, passes); }

// all `passes` digit histograms in one read of the keys
template <typename K>
__device__ __forceinline__ void sort_histogram_body(const K* __restrict__ keys, const unsigned int* __restrict__ n_ptr,
                                                    const SortScratch& s, int passes, unsigned int blk,
                                                    unsigned int nblk) {
    __shared__ unsigned int h[kSortMaxPasses][kRadix];
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

template <typename K>
__global__ void __launch_bounds__(kThreads) k_sort_histogram(const K* __restrict__ keys,
                                                             const unsigned int* __restrict__ n_ptr,
                                                             SortScratch s, int passes) {
    sort_histogram_body<K>(keys, n_ptr, s, passes, blockIdx.x, gridDim.x);
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
template <bool kWithValues, typename K, int kBits>
__device__ __forceinline__ void sort_pass_body(const K* __restrict__ keys_in, K* __restrict__ keys_out,
                                               const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ vals_out,
                                               const unsigned int* __restrict__ n_ptr, const SortScratch& s,
                                               int pass, unsigned int blk) {
    constexpr int R = 1 << kBits;
    constexpr int D = R / kThreads;
    constexpr int kLA = D == 1 ? kLookAhead : kLookAhead / 2;  // look-back words per digit and round
    static_assert(D >= 1 && D * kThreads == R, "whole digits per thread");
    __shared__ unsigned int warp_hist[kWarps][R + 1];  // last column: out-of-range keys
    __shared__ unsigned int digit_base[R];
    __shared__ unsigned int pass_offset[R];
    __shared__ unsigned int wsum[kWarps];
    __shared__ unsigned int tile_id;

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

template <bool kWithValues, typename K>
__global__ void __launch_bounds__(kThreads) k_sort_pass(const K* __restrict__ keys_in,
                                                        K* __restrict__ keys_out,
                                                        const uint32_t* __restrict__ vals_in,
                                                        uint32_t* __restrict__ vals_out,
                                                        const unsigned int* __restrict__ n_ptr,
                                                        SortScratch s, int pass) {
    sort_pass_body<kWithValues, K, 8>(keys_in, keys_out, vals_in, vals_out, n_ptr, s, pass, blockIdx.x);
}

// a pass of the frame keys' 10-bit digits
__global__ void __launch_bounds__(kThreads) k_sort_pass_frame(const uint32_t* __restrict__ keys_in,
                                                              uint32_t* __restrict__ keys_out,
                                                              const unsigned int* __restrict__ n_ptr,
                                                              SortScratch s, int pass) {
    sort_pass_body<false, uint32_t, kFrameDigitBits>(keys_in, keys_out, nullptr, nullptr, n_ptr, s, pass,
                                                     blockIdx.x);
}

// ---- batched: every volume of a batch sorts its frame's new keys, one
// launch per stage; a volume's CTAs take its tiles from its own counter
__global__ void k_sort_prepare_batch(const FuseJob* __restrict__ jobs, int n, int passes) {
    if ((int)blockIdx.x < n) sort_prepare_body(jobs[blockIdx.x].ss, passes);
}

template <typename K>
__global__ void __launch_bounds__(kThreads) k_sort_histogram_batch(const FuseJob* __restrict__ jobs, BlockMap m,
                                                                   int passes) {
    const int v = block_owner(m, blockIdx.x);
    const FuseJob& j = jobs[v];
    const unsigned int b0 = m.first[v];
    sort_histogram_body<K>((const K*)j.vb.new_keys, &j.ctl->n_new, j.ss, passes, blockIdx.x - b0,
                           m.first[v + 1] - b0);
}

template <typename K>
__global__ void __launch_bounds__(kThreads) k_sort_pass_batch(const FuseJob* __restrict__ jobs, BlockMap m,
                                                              int pass) {
    const int v = block_owner(m, blockIdx.x);
    const FuseJob& j = jobs[v];
    K* keys = (K*)j.vb.new_keys;
    K* alt = (K*)j.ss.alt_keys;
    // passes alternate between the new-key buffer and the sort's spare one
    sort_pass_body<false, K, 8>(pass & 1 ? alt : keys, pass & 1 ? keys : alt, nullptr, nullptr, &j.ctl->n_new,
                                j.ss, pass, blockIdx.x - m.first[v]);
}

// process-wide look-back limits (kifi_sort_set_fault_injection)
std::atomic<unsigned long long> g_spin_limit{kSpinLimit};
std::atomic<unsigned int> g_first_tile{0u};

}  // namespace

size_t sort_max_tiles(size_t max_n) { return (max_n + kTile - 1) / kTile + 1; }

cudaError_t sort_scratch_alloc(SortScratch* s, size_t max_n, cudaStream_t st) {
    *s = SortScratch{};
    s->max_tiles = sort_max_tiles(max_n);
    s->max_n = max_n;
    cudaError_t e;
    if ((e = cudaMalloc(&s->hist, kSortHistWords * sizeof(unsigned int) + 64))) return e;
    if ((e = cudaMalloc(&s->tile_counter, 8 * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&s->epoch, sizeof(unsigned long long)))) return e;
    if ((e = cudaMemsetAsync(s->epoch, 0, sizeof(unsigned long long), st))) return e;
    size_t lb = (size_t)kSortHistWords * s->max_tiles * sizeof(unsigned long long);
    if ((e = cudaMalloc(&s->lookback, lb))) return e;
    if ((e = cudaMemsetAsync(s->lookback, 0, lb, st))) return e;
    if ((e = cudaMalloc(&s->alt_keys, (max_n + 64) * sizeof(uint64_t)))) return e;
    if ((e = cudaMalloc(&s->alt_vals, (max_n + 64) * sizeof(uint32_t)))) return e;
    return cudaSuccess;
}

void sort_scratch_free(SortScratch* s) {
    cudaFree(s->hist);
    cudaFree(s->tile_counter);
    cudaFree(s->epoch);
    cudaFree(s->lookback);
    cudaFree(s->alt_keys);
    cudaFree(s->alt_vals);
    *s = SortScratch{};
}

template <typename K>
static cudaError_t sort_t(K* keys, int passes, uint32_t* vals, const unsigned int* n_dev, SortScratch& s,
                          unsigned int* status, int grid_ctas, cudaStream_t st) {
    s.status = status;
    s.spin_limit = g_spin_limit.load();
    s.first_tile = g_first_tile.load();
    k_sort_prepare<<<1, 256, 0, st>>>(s, passes);
    k_sort_histogram<K><<<grid_ctas, kThreads, 0, st>>>(keys, n_dev, s, passes);
    K *ki = keys, *ko = (K*)s.alt_keys;
    uint32_t *vi = vals, *vo = s.alt_vals;
    for (int pass = 0; pass < passes; ++pass) {
        if (vals)
            k_sort_pass<true, K><<<grid_ctas, kThreads, 0, st>>>(ki, ko, vi, vo, n_dev, s, pass);
        else
            k_sort_pass<false, K><<<grid_ctas, kThreads, 0, st>>>(ki, ko, nullptr, nullptr, n_dev, s, pass);
        K* t = ki;
        ki = ko;
        ko = t;
        uint32_t* tv = vi;
        vi = vo;
        vo = tv;
    }
    return cudaGetLastError();
}

void sort_limits(SortScratch* s) {
    s->spin_limit = g_spin_limit.load();
    s->first_tile = g_first_tile.load();
}

// keys -> alt -> keys -> alt: the sorted keys end in s.alt_keys
cudaError_t sort_frame_keys(uint32_t* keys, const unsigned int* n_dev, SortScratch& s, unsigned int* status,
                            int grid_ctas, cudaStream_t st, const uint32_t** sorted) {
    s.status = status;
    uint32_t* alt = (uint32_t*)s.alt_keys;
    for (int pass = 0; pass < kFrameSortPasses; ++pass)
        k_sort_pass_frame<<<grid_ctas, kThreads, 0, st>>>(pass & 1 ? alt : keys, pass & 1 ? keys : alt, n_dev, s,
                                                          pass);
    *sorted = kFrameSortPasses & 1 ? alt : keys;
    return cudaGetLastError();
}

template <typename K>
static cudaError_t sort_batch_t(const FuseJob* jobs, int n, int passes, const BlockMap& hist, const BlockMap& pass,
                                unsigned int hist_ctas, unsigned int pass_ctas, cudaStream_t st) {
    k_sort_prepare_batch<<<n, 256, 0, st>>>(jobs, n, passes);
    k_sort_histogram_batch<K><<<hist_ctas, kThreads, 0, st>>>(jobs, hist, passes);
    for (int p = 0; p < passes; ++p) k_sort_pass_batch<K><<<pass_ctas, kThreads, 0, st>>>(jobs, pass, p);
    return cudaGetLastError();
}

// Sorts keys[0..*n_dev) (and vals, when not null) in place.  *n_dev must not
// exceed s.max_n.  An even number of passes leaves the result in the
// caller's buffers.
cudaError_t sort_u32(uint32_t* keys, uint32_t* vals, const unsigned int* n_dev, SortScratch& s,
                     unsigned int* status, int grid_ctas, cudaStream_t st) {
    return sort_t<uint32_t>(keys, 4, vals, n_dev, s, status, grid_ctas, st);
}

cudaError_t sort_keys(void* keys, int key_bytes, int key_bits, uint32_t* vals, const unsigned int* n_dev,
                      SortScratch& s, unsigned int* status, int grid_ctas, cudaStream_t st) {
    int passes = (key_bits + 7) / 8;
    passes += passes & 1;
    if (passes < 2) passes = 2;
    if (key_bytes == 8)
        return sort_t<uint64_t>((uint64_t*)keys, passes > kSortMaxPasses ? kSortMaxPasses : passes, vals, n_dev, s,
                                status, grid_ctas, st);
    return sort_t<uint32_t>((uint32_t*)keys, passes > 4 ? 4 : passes, vals, n_dev, s, status, grid_ctas, st);
}

cudaError_t sort_batch_enqueue(const FuseJob* jobs, int n, int key_bytes, int passes, const BlockMap& hist,
                               const BlockMap& pass, cudaStream_t st) {
    if (key_bytes == 8) return sort_batch_t<uint64_t>(jobs, n, passes, hist, pass, hist.grid, pass.grid, st);
    return sort_batch_t<uint32_t>(jobs, n, passes, hist, pass, hist.grid, pass.grid, st);
}

}  // namespace kifi

extern "C" kifi_status kifi_sort_set_fault_injection(unsigned int skip_tiles, unsigned long long spin_limit) {
    kifi::g_first_tile.store(skip_tiles);
    kifi::g_spin_limit.store(spin_limit ? spin_limit : kifi::kSpinLimit);
    return KIFI_OK;
}
