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

#include "kifi_sort_body.cuh"

namespace kifi {
namespace {

using namespace sort_detail;

__global__ void k_sort_prepare(SortScratch s, int passes) { sort_prepare_body(s, passes); }

template <typename K>
__global__ void __launch_bounds__(kThreads) k_sort_histogram(const K* __restrict__ keys,
                                                             const unsigned int* __restrict__ n_ptr,
                                                             SortScratch s, int passes) {
    __shared__ SortHistSmem sm;
    sort_histogram_body<K>(keys, n_ptr, s, passes, blockIdx.x, gridDim.x, sm);
}

template <bool kWithValues, typename K>
__global__ void __launch_bounds__(kThreads) k_sort_pass(const K* __restrict__ keys_in,
                                                        K* __restrict__ keys_out,
                                                        const uint32_t* __restrict__ vals_in,
                                                        uint32_t* __restrict__ vals_out,
                                                        const unsigned int* __restrict__ n_ptr,
                                                        SortScratch s, int pass) {
    __shared__ SortPassSmem<8> sm;
    sort_pass_body<kWithValues, K, 8>(keys_in, keys_out, vals_in, vals_out, n_ptr, s, pass, blockIdx.x, sm);
}

// a pass of the frame keys' 10-bit digits
__global__ void __launch_bounds__(kThreads) k_sort_pass_frame(const uint32_t* __restrict__ keys_in,
                                                              uint32_t* __restrict__ keys_out,
                                                              const unsigned int* __restrict__ n_ptr,
                                                              SortScratch s, int pass) {
    __shared__ SortPassSmem<kFrameDigitBits> sm;
    sort_pass_body<false, uint32_t, kFrameDigitBits>(keys_in, keys_out, nullptr, nullptr, n_ptr, s, pass,
                                                     blockIdx.x, sm);
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
    __shared__ SortHistSmem sm;
    sort_histogram_body<K>((const K*)j.vb.new_keys, &j.ctl->n_new, j.ss, passes, blockIdx.x - b0,
                           m.first[v + 1] - b0, sm);
}

template <typename K>
__global__ void __launch_bounds__(kThreads) k_sort_pass_batch(const FuseJob* __restrict__ jobs, BlockMap m,
                                                              int pass) {
    const int v = block_owner(m, blockIdx.x);
    const FuseJob& j = jobs[v];
    K* keys = (K*)j.vb.new_keys;
    K* alt = (K*)j.ss.alt_keys;
    // passes alternate between the new-key buffer and the sort's spare one
    __shared__ SortPassSmem<8> sm;
    sort_pass_body<false, K, 8>(pass & 1 ? alt : keys, pass & 1 ? keys : alt, nullptr, nullptr, &j.ctl->n_new,
                                j.ss, pass, blockIdx.x - m.first[v], sm);
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
