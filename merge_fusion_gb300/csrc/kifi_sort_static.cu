// kifi_sort_static.cu -- kifi_radix_sort_pairs_u32_static: the library's
// radix sort (kifi_sort.cu) run on a device array in place, with every byte
// of scratch taken from one file-scope static __device__ array instead of
// cudaMalloc.  The call allocates nothing.
//
// Scratch layout (byte offsets into g_sort_scratch, 256-byte aligned):
//
//   0          generation counter of the look-back words (u64)   zero at load
//   8          device status word (u32)                          cleared per call
//   12         key count (u32)                                   written per call
//   256        dynamic tile counters, 8 x u32                    cleared per call
//   512        digit histograms, 4 x 256 x u32 (+64 B)           cleared per call
//   kLookback  look-back words, 4 x kTiles x 256 x u64           zero at load
//   kAltKeys   ping-pong keys,   (kMaxKeys + 64) x u32
//   kAltVals   ping-pong values, (kMaxKeys + 64) x u32
//
// What must start at zero: the generation counter and the look-back words.
// Each sort bumps the counter and tags its look-back words with it, so words
// left by an earlier sort are ignored without clearing -- provided no word
// ever carries a tag the counter has not reached yet.  Static device memory
// is zero-initialised when the module is loaded, which gives exactly that.
// Everything else is (re)initialised by every call before it is read.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and the SM count, and
// caches both per device; later calls only read the cache.
//
// One scratch area per device: two calls that overlap in time race on it.
#include <cstdio>
#include <mutex>

#include "kifi_api_util.h"

namespace kifi {
namespace {

constexpr size_t kMaxKeys = (size_t)KIFI_RADIX_SORT_STATIC_MAX;
constexpr size_t kSortTile = 2048;  // keys per tile of k_sort_pass
constexpr size_t kTiles = (kMaxKeys + kSortTile - 1) / kSortTile + 1;
constexpr size_t kLookback = 5120;
constexpr size_t kAltKeys = kLookback + 4 * kTiles * 256 * sizeof(unsigned long long);
constexpr size_t kAltVals = kAltKeys + ((kMaxKeys + 64) * sizeof(uint32_t) + 255) / 256 * 256;
constexpr size_t kScratchBytes = kAltVals + ((kMaxKeys + 64) * sizeof(uint32_t) + 255) / 256 * 256;
static_assert(512 + 4 * 256 * sizeof(unsigned int) + 64 <= kLookback, "histograms overlap the look-back words");

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
struct DeviceScratch {
    bool ready = false;
    unsigned char* base = nullptr;
    int sort_ctas = 0;
};
std::mutex g_setup_mutex;
DeviceScratch g_devices[kMaxDevices];

kifi_status scratch_for_current_device(const DeviceScratch** out) {
    int dev = 0;
    KIFI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(KIFI_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceScratch& d = g_devices[dev];
    if (!d.ready) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the static sort scratch");
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
        d.base = (unsigned char*)p;
        d.sort_ctas = 4 * sms;
        d.ready = true;
    }
    *out = &d;
    return KIFI_OK;
}

__global__ void k_static_sort_begin(unsigned int* count, unsigned int* status, unsigned int n) {
    *count = n;
    *status = 0u;
}

}  // namespace
}  // namespace kifi

using namespace kifi;

extern "C" kifi_status kifi_radix_sort_pairs_u32_static(uint32_t* keys_dev, uint32_t* values_dev, size_t n,
                                                         void* stream) {
    if (n == 0) return KIFI_OK;
    if (!keys_dev) return fail(KIFI_ERR_INVALID_ARGUMENT, "null keys");
    if (n > kMaxKeys) {
        char msg[160];
        std::snprintf(msg, sizeof msg,
                      "kifi_radix_sort_pairs_u32_static: n = %zu exceeds the static scratch limit of %zu keys",
                      n, kMaxKeys);
        return fail(KIFI_ERR_INVALID_ARGUMENT, msg);
    }
    if (sort_max_tiles(n) > kTiles) return fail(KIFI_ERR_UNSUPPORTED, "static sort scratch too small");
    const DeviceScratch* d = nullptr;
    kifi_status s = scratch_for_current_device(&d);
    if (s) return s;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* b = d->base;
    SortScratch ss;
    ss.epoch = (unsigned long long*)b;
    ss.tile_counter = (unsigned int*)(b + 256);
    ss.hist = (unsigned int*)(b + 512);
    ss.lookback = (unsigned long long*)(b + kLookback);
    ss.alt_keys = (uint32_t*)(b + kAltKeys);
    ss.alt_vals = (uint32_t*)(b + kAltVals);
    ss.max_tiles = kTiles;
    ss.max_n = kMaxKeys;
    unsigned int* status = (unsigned int*)(b + 8);
    unsigned int* count = (unsigned int*)(b + 12);
    k_static_sort_begin<<<1, 1, 0, st>>>(count, status, (unsigned int)n);
    KIFI_CUDA(cudaGetLastError());
    KIFI_CUDA(sort_u32(keys_dev, values_dev, count, ss, status, d->sort_ctas, st));
    unsigned int h_status = 0;
    KIFI_CUDA(cudaMemcpyAsync(&h_status, status, sizeof h_status, cudaMemcpyDeviceToHost, st));
    KIFI_CUDA(cudaStreamSynchronize(st));
    if (h_status & KIFI_DEV_ERR_TIMEOUT) return fail(KIFI_ERR_TIMEOUT, "a bounded device wait gave up");
    return KIFI_OK;
}
