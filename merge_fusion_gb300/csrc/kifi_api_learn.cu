// kifi_api_learn.cu -- C ABI of the learned pose proposer's tensor-core
// building blocks (no counterpart in the reference).
#include <mutex>

#include "kifi_api_util.h"

using namespace kifi;

namespace {
// where the GEMM's bounded waits report; one per device, shared by every
// call of kifi_gemm_bf16 and kifi_conv3x3s2_bf16 (overlapping calls race on
// it, as the header says)
__device__ unsigned int g_gemm_status;
}

extern "C" {

kifi_status kifi_gemm_bf16(const void* a_dev, const void* b_dev, float* c_dev, int m, int n, int k, int lda,
                           int ldb, int ldc, int k_split, int accumulate, void* stream) {
    if (!a_dev || !b_dev || !c_dev || m < 0 || n < 0 || k < 0) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    if (k % 8 || lda % 8 || ldb % 8 || (k_split > 0 && k_split % 8) || ((uintptr_t)a_dev | (uintptr_t)b_dev) % 16 ||
        lda < k || ldb < k || ldc < n)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "gemm: K, lda, ldb and the split must be multiples of 8, "
                                                "operands 16-byte aligned");
    if (k_split > 0 && k_split < k && !accumulate)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "gemm: a split K accumulates into C");
    if (m == 0 || n == 0) return KIFI_OK;
    unsigned int* status = nullptr;
    KIFI_CUDA(cudaGetSymbolAddress((void**)&status, g_gemm_status));
    cudaStream_t st = (cudaStream_t)stream;
    KIFI_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned int), st));
    KIFI_CUDA(gemm_bf16_enqueue(a_dev, b_dev, c_dev, m, n, k, lda, ldb, ldc, k_split, accumulate != 0, status, st));
    unsigned int h = 0;
    KIFI_CUDA(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, st));
    KIFI_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(KIFI_ERR_TIMEOUT, "gemm: a bounded device wait gave up");
    return KIFI_OK;
}

kifi_status kifi_conv3x3s2_bf16(const void* x_dev, int batch, int height, int width, int cin, const void* w_dev,
                                int cout, int kp, const float* bias_dev, int relu, void* out_dev, void* stream) {
    if (!x_dev || !w_dev || !out_dev || batch < 0 || height <= 0 || width <= 0)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    if ((cin != 32 && cin != 64) || (cout != 64 && cout != 128) || kp < 9 * cin || kp % 8 ||
        ((uintptr_t)x_dev | (uintptr_t)w_dev | (uintptr_t)out_dev) % 16 || (width + 1) / 2 > 128)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "conv: cin 32 or 64, cout 64 or 128, kp >= 9 cin and a multiple "
                                                "of 8, output width <= 128, 16-byte aligned buffers");
    if (batch == 0) return KIFI_OK;
    unsigned int* status = nullptr;
    KIFI_CUDA(cudaGetSymbolAddress((void**)&status, g_gemm_status));
    cudaStream_t st = (cudaStream_t)stream;
    KIFI_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned int), st));
    KIFI_CUDA(conv3x3s2_bf16_enqueue(x_dev, batch, height, width, cin, w_dev, cout, kp, bias_dev, relu != 0, out_dev,
                                     status, st));
    unsigned int h = 0;
    KIFI_CUDA(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, st));
    KIFI_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(KIFI_ERR_TIMEOUT, "conv: a bounded device wait gave up");
    return KIFI_OK;
}

}  // extern "C"
