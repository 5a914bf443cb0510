// kifi_proposer.cu -- the learned ICP pose proposer: a small convolutional
// network that maps two box-downsampled depth frames (2 x 60 x 80, FP16,
// metres, 0 = no depth) to a 6-DoF twist that warm-starts ICP.  No
// counterpart in the reference.
//
//   conv 3x3/2 2->32, ReLU     60x80 -> 30x40
//   conv 3x3/2 32->64, ReLU    -> 15x20
//   conv 3x3/2 64->64, ReLU    -> 8x10
//   conv 3x3/2 64->128, ReLU   -> 4x5
//   global average pool        -> 128
//   fc 128->64, ReLU; fc 64->6
//
// Activations are NHWC BF16; every product -- convolutions 2-4 as implicit
// GEMMs whose A tiles TMA gathers straight from the previous activation,
// convolution 1 through its im2col matrix, the fully connected layers, and
// all the backward products -- runs on the TMA-fed tcgen05 GEMM
// (kifi_tc_gemm.cu) with FP32 accumulation; forward products add the bias
// and apply the ReLU in the GEMM epilogue.  Parameters keep an
// FP32 master copy updated by Adam, which also writes the BF16 copies the
// GEMMs read.  Padded parameter entries (conv 1's K = 18 padded to 32, the
// output layer's 6 rows padded to 16) stay zero.
//
// Backward products, with col the im2col matrix [M x Kp] and dY the
// pre-activation gradient [M x Cout]:
//   dW    [Cout x Kp] = dY^T col      A = dY^T, B = col^T (inner M, split K)
//   dcol  [M x Kp]    = dY W          A = dY,   B = W^T
//   dX                = col2im(dcol)  a gather over the <= 4 taps per input
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "kifi_api_util.h"

using namespace kifi;

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kInH = 60, kInW = 80, kInC = 2;
constexpr int kConvs = 4;
constexpr int kCin[kConvs] = {2, 32, 64, 64};
constexpr int kCout[kConvs] = {32, 64, 64, 128};
constexpr int kHin[kConvs] = {60, 30, 15, 8};
constexpr int kWin[kConvs] = {80, 40, 20, 10};
constexpr int kHout[kConvs] = {30, 15, 8, 4};
constexpr int kWout[kConvs] = {40, 20, 10, 5};
constexpr int kKp[kConvs] = {32, 288, 576, 576};  // 9 * Cin, padded to a multiple of 16
constexpr int kFc1 = 64, kOut = 6, kOutPad = 16;
constexpr int kThreads = 256;

// parameter tensors, in order: conv W/b x 4, fc1 W/b, fc2 W/b
struct Layout {
    size_t off[12], size[12], total;
    Layout() {
        const size_t sz[12] = {32 * 32, 32, 64 * 288, 64, 64 * 576, 64, 128 * 576, 128, 64 * 128, 64,
                               16 * 64, 16};
        total = 0;
        for (int i = 0; i < 12; ++i) {
            off[i] = total;
            size[i] = sz[i];
            total += (sz[i] + 7) / 8 * 8;  // 16-byte aligned BF16 copies
        }
    }
};
const Layout kLayout;

int blocks(size_t n) { return (int)((n + kThreads - 1) / kThreads); }

// ------------------------------------------------------------------ kernels

// Box mean of the valid (non-zero) depth of each 8x8 block of two frames ->
// NHWC FP16 [60][80][2]; 0 where a block has no depth.
__global__ void k_downsample(const void* __restrict__ da, const void* __restrict__ db, int u16, int width,
                             int height, __half* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kInH * kInW * 2) return;
    const int f = i & 1, px = (i >> 1) % kInW, py = (i >> 1) / kInW;
    const void* d = f ? db : da;
    const int bw = width / kInW, bh = height / kInH;
    float sum = 0.0f;
    int n = 0;
    for (int y = py * bh; y < (py + 1) * bh; ++y)
        for (int x = px * bw; x < (px + 1) * bw; ++x) {
            const size_t at = (size_t)y * width + x;
            const float z = u16 ? fmul((float)((const unsigned short*)d)[at], 0.001f) : ((const float*)d)[at];
            if (z > 0.0f) {
                sum += z;
                ++n;
            }
        }
    out[i] = __float2half_rn(n ? sum / (float)n : 0.0f);
}

// im2col of a 3x3, stride 2, pad 1 convolution: col[m][k], m = (b, oy, ox),
// k = (ky * 3 + kx) * C + c, zero outside the input and for k >= 9C
template <typename T>
__global__ void k_im2col(const T* __restrict__ x, int batch, int H, int W, int C, int Ho, int Wo, int Kp,
                         bf16* __restrict__ col) {
    const size_t n = (size_t)batch * Ho * Wo * Kp;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(i % Kp);
        const size_t m = i / Kp;
        const int ox = (int)(m % Wo), oy = (int)((m / Wo) % Ho), b = (int)(m / ((size_t)Wo * Ho));
        float v = 0.0f;
        if (k < 9 * C) {
            const int c = k % C, tap = k / C, ky = tap / 3, kx = tap % 3;
            const int iy = 2 * oy - 1 + ky, ix = 2 * ox - 1 + kx;
            if (iy >= 0 && iy < H && ix >= 0 && ix < W) v = (float)x[(((size_t)b * H + iy) * W + ix) * C + c];
        }
        col[i] = __float2bfloat16_rn(v);
    }
}

// out[c][r] = in[r][c], 32x32 tiles through shared memory
__global__ void k_transpose(const bf16* __restrict__ in, int R, int Cc, bf16* __restrict__ out) {
    __shared__ bf16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        if (r < R && c < Cc) t[j][threadIdx.x] = in[(size_t)r * Cc + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (r < R && c < Cc) out[(size_t)c * R + r] = t[threadIdx.x][j];
    }
}

// global average pool: [B][P][C] -> [B][C]
__global__ void k_gap(const bf16* __restrict__ act, int batch, int P, int C, bf16* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch * C) return;
    const int b = i / C, c = i % C;
    float s = 0.0f;
    for (int p = 0; p < P; ++p) s += __bfloat162float(act[((size_t)b * P + p) * C + c]);
    out[i] = __float2bfloat16_rn(s / (float)P);
}

// mean squared error over batch x 6; d = dL/dpred into dpred[B][16] (FP32
// and BF16), columns 6..15 zero; the summed loss is added to *loss
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target, int batch,
                      float* __restrict__ dpred, bf16* __restrict__ dpred_bf, float* __restrict__ loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < batch * kOutPad) {
        const int b = i / kOutPad, j = i % kOutPad;
        float d = 0.0f;
        if (j < kOut) {
            const float e = pred[i] - target[b * kOut + j];
            l = e * e;
            d = 2.0f * e / (float)(batch * kOut);
        }
        dpred[i] = d;
        dpred_bf[i] = __float2bfloat16_rn(d);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0f) atomicAdd(loss, l / (float)(batch * kOut));
}

// column sums of g [M][C] (FP32) into db[C] (+=)
__global__ void k_colsum(const float* __restrict__ g, int M, int C, float* __restrict__ db) {
    const int c = blockIdx.x;
    float s = 0.0f;
    for (int m = threadIdx.x; m < M; m += blockDim.x) s += g[(size_t)m * C + c];
    __shared__ float red[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) t += red[w];
        db[c] += t;
    }
}

// ReLU backward: g = act > 0 ? g : 0 (in place, FP32) and a BF16 copy
__global__ void k_relu_back(float* __restrict__ g, const bf16* __restrict__ act, size_t n, bf16* __restrict__ gb) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float v = __bfloat162float(act[i]) > 0.0f ? g[i] : 0.0f;
        g[i] = v;
        gb[i] = __float2bfloat16_rn(v);
    }
}

// global average pool backward: d[B][P][C] = dg[B][C] / P
__global__ void k_gap_back(const float* __restrict__ dg, int batch, int P, int C, float* __restrict__ d) {
    const size_t n = (size_t)batch * P * C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int b = (int)(i / ((size_t)P * C));
        d[i] = dg[(size_t)b * C + c] / (float)P;
    }
}

// col2im of the 3x3 / stride 2 / pad 1 convolution as a gather: input
// element (b, iy, ix, c) collects dcol[(b, oy, ox)][(ky, kx, c)] over the taps
// with iy = 2 oy - 1 + ky, ix = 2 ox - 1 + kx
__global__ void k_col2im(const float* __restrict__ dcol, int batch, int H, int W, int C, int Ho, int Wo, int Kp,
                         float* __restrict__ dx) {
    const size_t n = (size_t)batch * H * W * C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int ix = (int)((i / C) % W), iy = (int)((i / ((size_t)C * W)) % H);
        const int b = (int)(i / ((size_t)C * W * H));
        float s = 0.0f;
        for (int ky = 0; ky < 3; ++ky) {
            const int ty = iy + 1 - ky;
            if (ty < 0 || (ty & 1) || (ty >> 1) >= Ho) continue;
            for (int kx = 0; kx < 3; ++kx) {
                const int tx = ix + 1 - kx;
                if (tx < 0 || (tx & 1) || (tx >> 1) >= Wo) continue;
                const size_t m = ((size_t)b * Ho + (ty >> 1)) * Wo + (tx >> 1);
                s += dcol[m * Kp + (ky * 3 + kx) * C + c];
            }
        }
        dx[i] = s;
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters; masked entries stay
// zero; writes the BF16 copies
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, const unsigned char* __restrict__ mask, size_t n, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, bf16* __restrict__ pb) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = 0.0f;
        if (mask[i]) {
            const float gi = g[i];
            const float a = b1 * m1[i] + (1.0f - b1) * gi;
            const float s = b2 * m2[i] + (1.0f - b2) * gi * gi;
            m1[i] = a;
            m2[i] = s;
            v = p[i] - lr * (a / bc1) / (sqrtf(s / bc2) + eps);
        }
        p[i] = v;
        pb[i] = __float2bfloat16_rn(v);
    }
}

__global__ void k_to_bf16(const float* __restrict__ p, size_t n, bf16* __restrict__ pb) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        pb[i] = __float2bfloat16_rn(p[i]);
}

}  // namespace

struct kifi_proposer {
    int device = 0, max_batch = 0;
    cudaStream_t stream = nullptr;
    unsigned int* status = nullptr;  // GEMM wait status
    float* loss = nullptr;
    // parameters (FP32 master, gradients, Adam moments), BF16 copies, trainable mask
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
    bf16* pb = nullptr;
    unsigned char* mask = nullptr;
    long long step = 0;
    // activations and scratch
    __half* x = nullptr;                 // the network input [B][60][80][2]
    bf16* col[kConvs] = {};              // im2col [M][Kp]
    bf16* colT[kConvs] = {};             // its transpose [Kp][M] (training)
    float* y = nullptr;                  // GEMM output / gradient scratch, FP32 (largest [M][C])
    float* y2 = nullptr;                 // second FP32 scratch (dcol, dX)
    bf16* act[kConvs] = {};              // conv activations [M][Cout]
    bf16 *gap = nullptr, *gapT = nullptr;   // [B][128], [128][B]
    bf16 *h1 = nullptr, *h1T = nullptr;     // [B][64], [64][B]
    float* out = nullptr;                   // [B][16]
    bf16 *dbf = nullptr, *dbfT = nullptr;   // BF16 gradient [M][C] and transpose
    bf16* wT = nullptr;                     // transposed weights
};

namespace {

size_t conv_m(int l, int batch) { return (size_t)batch * kHout[l] * kWout[l]; }

kifi_status gemm(kifi_proposer* pr, const void* A, const void* B, float* C, int M, int N, int K, int lda, int ldb,
                 int ldc, int k_split, bool acc, const GemmEpilogue* epi = nullptr) {
    KIFI_CUDA(gemm_bf16_enqueue(A, B, C, M, N, K, lda, ldb, ldc, k_split, acc, pr->status, pr->stream, epi));
    return KIFI_OK;
}
kifi_status transpose(kifi_proposer* pr, const bf16* in, int R, int Cc, bf16* out) {
    dim3 grid((Cc + 31) / 32, (R + 31) / 32);
    k_transpose<<<grid, dim3(32, 8), 0, pr->stream>>>(in, R, Cc, out);
    KIFI_CUDA(cudaGetLastError());
    return KIFI_OK;
}

const bf16* wb(const kifi_proposer* pr, int t) { return pr->pb + kLayout.off[t]; }
const float* pf(const kifi_proposer* pr, int t) { return pr->p + kLayout.off[t]; }
float* gf(kifi_proposer* pr, int t) { return pr->g + kLayout.off[t]; }

// forward pass; with `train` the transposed im2col matrices are kept for the
// weight gradients.  Convolutions 2-4 run as implicit GEMMs over the previous
// activation; convolution 1 (Cin = 2) through its im2col matrix.  Bias and
// ReLU are applied in the GEMM epilogue, which writes the BF16 activation.
kifi_status forward(kifi_proposer* pr, int batch, bool train) {
    kifi_status s;
    cudaStream_t st = pr->stream;
    const int grid = pr->max_batch > 0 ? 4 * 152 : 1;
    for (int l = 0; l < kConvs; ++l) {
        const int M = (int)conv_m(l, batch);
        if (l == 0)
            k_im2col<__half><<<grid, kThreads, 0, st>>>(pr->x, batch, kHin[0], kWin[0], kCin[0], kHout[0],
                                                        kWout[0], kKp[0], pr->col[0]);
        else if (train)
            k_im2col<bf16><<<grid, kThreads, 0, st>>>(pr->act[l - 1], batch, kHin[l], kWin[l], kCin[l], kHout[l],
                                                      kWout[l], kKp[l], pr->col[l]);
        KIFI_CUDA(cudaGetLastError());
        if (train && (s = transpose(pr, pr->col[l], M, kKp[l], pr->colT[l]))) return s;
        GemmEpilogue epi;
        epi.bias = pf(pr, 2 * l + 1);
        epi.relu = true;
        epi.out_bf16 = pr->act[l];
        if (l == 0) {
            if ((s = gemm(pr, pr->col[0], wb(pr, 0), nullptr, M, kCout[0], kKp[0], kKp[0], kKp[0], kCout[0], 0, false,
                          &epi)))
                return s;
        } else {
            KIFI_CUDA(conv3x3s2_bf16_enqueue(pr->act[l - 1], batch, kHin[l], kWin[l], kCin[l], wb(pr, 2 * l),
                                             kCout[l], kKp[l], epi.bias, true, pr->act[l], pr->status, st));
        }
    }
    k_gap<<<blocks((size_t)batch * 128), kThreads, 0, st>>>(pr->act[3], batch, kHout[3] * kWout[3], 128, pr->gap);
    GemmEpilogue e1;
    e1.bias = pf(pr, 9);
    e1.relu = true;
    e1.out_bf16 = pr->h1;
    if ((s = gemm(pr, pr->gap, wb(pr, 8), nullptr, batch, kFc1, 128, 128, 128, kFc1, 0, false, &e1))) return s;
    GemmEpilogue e2;
    e2.bias = pf(pr, 11);
    if ((s = gemm(pr, pr->h1, wb(pr, 10), pr->out, batch, kOutPad, kFc1, kFc1, kFc1, kOutPad, 0, false, &e2)))
        return s;
    KIFI_CUDA(cudaGetLastError());
    return KIFI_OK;
}

// backward pass from dL/dout (FP32 in pr->y2 [B][16], BF16 in pr->dbf) into pr->g
kifi_status backward(kifi_proposer* pr, int batch) {
    kifi_status s;
    cudaStream_t st = pr->stream;
    const int grid = 4 * 152;
    KIFI_CUDA(cudaMemsetAsync(pr->g, 0, kLayout.total * sizeof(float), st));
    // fc2: dW2 [16 x 64] = dout^T h1, db2 = colsum(dout), dh1 = dout W2
    if ((s = transpose(pr, pr->dbf, batch, kOutPad, pr->dbfT))) return s;
    if ((s = transpose(pr, pr->h1, batch, kFc1, pr->h1T))) return s;
    if ((s = gemm(pr, pr->dbfT, pr->h1T, gf(pr, 10), kOutPad, kFc1, batch, batch, batch, kFc1, batch, true)))
        return s;
    k_colsum<<<kOutPad, kThreads, 0, st>>>(pr->y2, batch, kOutPad, gf(pr, 11));
    if ((s = transpose(pr, wb(pr, 10), kOutPad, kFc1, pr->wT))) return s;
    if ((s = gemm(pr, pr->dbf, pr->wT, pr->y, batch, kFc1, kOutPad, kOutPad, kOutPad, kFc1, 0, false))) return s;
    k_relu_back<<<blocks((size_t)batch * kFc1), kThreads, 0, st>>>(pr->y, pr->h1, (size_t)batch * kFc1, pr->dbf);
    // fc1: dW1 [64 x 128] = dh^T gap, db1, dgap = dh W1
    if ((s = transpose(pr, pr->dbf, batch, kFc1, pr->dbfT))) return s;
    if ((s = transpose(pr, pr->gap, batch, 128, pr->gapT))) return s;
    if ((s = gemm(pr, pr->dbfT, pr->gapT, gf(pr, 8), kFc1, 128, batch, batch, batch, 128, batch, true))) return s;
    k_colsum<<<kFc1, kThreads, 0, st>>>(pr->y, batch, kFc1, gf(pr, 9));
    if ((s = transpose(pr, wb(pr, 8), kFc1, 128, pr->wT))) return s;
    if ((s = gemm(pr, pr->dbf, pr->wT, pr->y2, batch, 128, kFc1, kFc1, kFc1, 128, 0, false))) return s;
    // pool backward into the last conv's gradient
    k_gap_back<<<grid, kThreads, 0, st>>>(pr->y2, batch, kHout[3] * kWout[3], 128, pr->y);
    for (int l = kConvs - 1; l >= 0; --l) {
        const int M = (int)conv_m(l, batch), Co = kCout[l], Kp = kKp[l];
        // pr->y holds dL/d(act l) [M][Co]: through the ReLU
        k_relu_back<<<grid, kThreads, 0, st>>>(pr->y, pr->act[l], (size_t)M * Co, pr->dbf);
        k_colsum<<<Co, kThreads, 0, st>>>(pr->y, M, Co, gf(pr, 2 * l + 1));
        if ((s = transpose(pr, pr->dbf, M, Co, pr->dbfT))) return s;
        // dW [Co x Kp] = dY^T col, inner M split across CTAs
        if ((s = gemm(pr, pr->dbfT, pr->colT[l], gf(pr, 2 * l), Co, Kp, M, M, M, Kp, 4096, true))) return s;
        if (l == 0) break;
        // dcol = dY W, then col2im into dL/d(act l-1)
        if ((s = transpose(pr, wb(pr, 2 * l), Co, Kp, pr->wT))) return s;
        if ((s = gemm(pr, pr->dbf, pr->wT, pr->y2, M, Kp, Co, Co, Co, Kp, 0, false))) return s;
        k_col2im<<<grid, kThreads, 0, st>>>(pr->y2, batch, kHin[l], kWin[l], kCin[l], kHout[l], kWout[l], Kp,
                                            pr->y);
    }
    KIFI_CUDA(cudaGetLastError());
    return KIFI_OK;
}

kifi_status take_status(kifi_proposer* pr) {
    unsigned int h = 0;
    KIFI_CUDA(cudaMemcpyAsync(&h, pr->status, sizeof h, cudaMemcpyDeviceToHost, pr->stream));
    KIFI_CUDA(cudaStreamSynchronize(pr->stream));
    if (h) {
        KIFI_CUDA(cudaMemsetAsync(pr->status, 0, sizeof(unsigned int), pr->stream));
        return fail(KIFI_ERR_TIMEOUT, "proposer: a bounded device wait gave up");
    }
    return KIFI_OK;
}

kifi_status check_batch(kifi_proposer* pr, int batch) {
    if (batch <= 0 || batch > pr->max_batch || batch % 8)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "proposer batch must be a positive multiple of 8 up to max_batch");
    return KIFI_OK;
}

}  // namespace

extern "C" {

kifi_status kifi_proposer_destroy(kifi_proposer* pr) {
    if (!pr) return KIFI_OK;
    if (pr->stream) cudaStreamSynchronize(pr->stream);
    void* bufs[] = {pr->status, pr->loss, pr->p, pr->g, pr->m1, pr->m2, pr->pb, pr->mask, pr->x, pr->y, pr->y2,
                    pr->gap, pr->gapT, pr->h1, pr->h1T, pr->out, pr->dbf, pr->dbfT, pr->wT};
    for (void* b : bufs) cudaFree(b);
    for (int l = 0; l < kConvs; ++l) {
        cudaFree(pr->col[l]);
        cudaFree(pr->colT[l]);
        cudaFree(pr->act[l]);
    }
    if (pr->stream) cudaStreamDestroy(pr->stream);
    delete pr;
    return KIFI_OK;
}

kifi_status kifi_proposer_create(int device, int max_batch, kifi_proposer** out) {
    if (!out || max_batch <= 0 || max_batch % 8) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    *out = nullptr;
    kifi_proposer* pr = new (std::nothrow) kifi_proposer();
    if (!pr) return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    pr->device = device;
    pr->max_batch = max_batch;
    const size_t B = (size_t)max_batch, P = kLayout.total;
    cudaError_t e = cudaSetDevice(device);
    if (!e) e = cudaStreamCreateWithFlags(&pr->stream, cudaStreamNonBlocking);
    auto alloc = [&](auto** ptr, size_t bytes) {
        if (!e) e = cudaMalloc((void**)ptr, bytes);
    };
    alloc(&pr->status, 16);
    alloc(&pr->loss, 16);
    alloc(&pr->p, P * 4);
    alloc(&pr->g, P * 4);
    alloc(&pr->m1, P * 4);
    alloc(&pr->m2, P * 4);
    alloc(&pr->pb, P * 2);
    alloc(&pr->mask, P);
    alloc(&pr->x, B * kInH * kInW * kInC * 2);
    size_t ymax = 0, colmax = 0, dmax = 0;
    for (int l = 0; l < kConvs; ++l) {
        const size_t M = conv_m(l, max_batch);
        alloc(&pr->col[l], M * kKp[l] * 2);
        alloc(&pr->colT[l], M * kKp[l] * 2);
        alloc(&pr->act[l], M * kCout[l] * 2);
        ymax = std::max(ymax, M * (size_t)kCout[l]);
        colmax = std::max(colmax, M * (size_t)kKp[l]);
        dmax = std::max(dmax, M * (size_t)kCout[l]);
        if (l > 0) ymax = std::max(ymax, (size_t)max_batch * kHin[l] * kWin[l] * kCin[l]);
    }
    alloc(&pr->y, ymax * 4);
    alloc(&pr->y2, std::max(colmax, B * 128) * 4);
    alloc(&pr->gap, B * 128 * 2);
    alloc(&pr->gapT, B * 128 * 2);
    alloc(&pr->h1, B * kFc1 * 2);
    alloc(&pr->h1T, B * kFc1 * 2);
    alloc(&pr->out, B * kOutPad * 4);
    alloc(&pr->dbf, dmax * 2);
    alloc(&pr->dbfT, dmax * 2);
    alloc(&pr->wT, 128 * 576 * 2);
    if (!e) e = cudaMemsetAsync(pr->status, 0, 16, pr->stream);
    if (!e) e = cudaMemsetAsync(pr->p, 0, P * 4, pr->stream);
    if (!e) e = cudaMemsetAsync(pr->m1, 0, P * 4, pr->stream);
    if (!e) e = cudaMemsetAsync(pr->m2, 0, P * 4, pr->stream);
    if (!e) e = cudaMemsetAsync(pr->pb, 0, P * 2, pr->stream);
    if (!e) {  // trainable mask: everything but the padding
        std::vector<unsigned char> m(P, 0);
        for (int t = 0; t < 12; ++t)
            for (size_t i = 0; i < kLayout.size[t]; ++i) {
                bool on = true;
                if (t == 0) on = (i % 32) < 18;         // conv 1: K = 18 of 32
                if (t == 10) on = (i / kFc1) < kOut;    // output rows 0..5
                if (t == 11) on = i < (size_t)kOut;
                m[kLayout.off[t] + i] = on ? 1 : 0;
            }
        // on the proposer's stream (non-blocking: it would not wait for the legacy default stream)
        e = cudaMemcpyAsync(pr->mask, m.data(), P, cudaMemcpyHostToDevice, pr->stream);
        if (!e) e = cudaStreamSynchronize(pr->stream);
    }
    if (e) {
        kifi_proposer_destroy(pr);
        return cuda_fail(e, "proposer allocation");
    }
    *out = pr;
    return KIFI_OK;
}

kifi_status kifi_proposer_param_count(kifi_proposer* pr, size_t* n) {
    if (!pr || !n) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *n = kLayout.total;
    return KIFI_OK;
}

kifi_status kifi_proposer_set_params(kifi_proposer* pr, const float* host, size_t n) {
    if (!pr || !host || n != kLayout.total) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad parameter vector");
    KIFI_CUDA(cudaSetDevice(pr->device));
    KIFI_CUDA(cudaMemcpyAsync(pr->p, host, n * 4, cudaMemcpyHostToDevice, pr->stream));
    k_to_bf16<<<blocks(n), kThreads, 0, pr->stream>>>(pr->p, n, pr->pb);
    KIFI_CUDA(cudaMemsetAsync(pr->m1, 0, n * 4, pr->stream));
    KIFI_CUDA(cudaMemsetAsync(pr->m2, 0, n * 4, pr->stream));
    pr->step = 0;
    KIFI_CUDA(cudaStreamSynchronize(pr->stream));
    return KIFI_OK;
}

kifi_status kifi_proposer_get_params(kifi_proposer* pr, float* host, size_t n) {
    if (!pr || !host || n != kLayout.total) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad parameter vector");
    KIFI_CUDA(cudaSetDevice(pr->device));
    KIFI_CUDA(cudaMemcpyAsync(host, pr->p, n * 4, cudaMemcpyDeviceToHost, pr->stream));
    KIFI_CUDA(cudaStreamSynchronize(pr->stream));
    return KIFI_OK;
}

kifi_status kifi_proposer_make_input(kifi_proposer* pr, const void* depth_a_dev, const void* depth_b_dev,
                                     int depth_is_u16, int width, int height, void* out_fp16_dev) {
    if (!pr || !depth_a_dev || !depth_b_dev || !out_fp16_dev || width % kInW || height % kInH || width <= 0 ||
        height <= 0)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument (frames must be multiples of 80 x 60)");
    KIFI_CUDA(cudaSetDevice(pr->device));
    k_downsample<<<blocks(kInH * kInW * 2), kThreads, 0, pr->stream>>>(depth_a_dev, depth_b_dev, depth_is_u16,
                                                                       width, height, (__half*)out_fp16_dev);
    KIFI_CUDA(cudaGetLastError());
    KIFI_CUDA(cudaStreamSynchronize(pr->stream));
    return KIFI_OK;
}

kifi_status kifi_proposer_set_inputs(kifi_proposer* pr, const void* inputs_fp16_dev, int batch) {
    if (!pr || !inputs_fp16_dev) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    kifi_status s = check_batch(pr, batch);
    if (s) return s;
    KIFI_CUDA(cudaSetDevice(pr->device));
    KIFI_CUDA(cudaMemcpyAsync(pr->x, inputs_fp16_dev, (size_t)batch * kInH * kInW * kInC * 2,
                              cudaMemcpyDeviceToDevice, pr->stream));
    return KIFI_OK;
}

kifi_status kifi_proposer_get_inputs(kifi_proposer* pr, void* out_fp16_dev, int batch) {
    if (!pr || !out_fp16_dev) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    kifi_status s = check_batch(pr, batch);
    if (s) return s;
    KIFI_CUDA(cudaSetDevice(pr->device));
    KIFI_CUDA(cudaMemcpyAsync(out_fp16_dev, pr->x, (size_t)batch * kInH * kInW * kInC * 2,
                              cudaMemcpyDeviceToDevice, pr->stream));
    KIFI_CUDA(cudaStreamSynchronize(pr->stream));
    return KIFI_OK;
}

kifi_status kifi_proposer_predict(kifi_proposer* pr, int batch, float* out_twists_host) {
    if (!pr || !out_twists_host) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    kifi_status s = check_batch(pr, batch);
    if (s) return s;
    KIFI_CUDA(cudaSetDevice(pr->device));
    if ((s = forward(pr, batch, false))) return s;
    std::vector<float> o((size_t)batch * kOutPad);
    KIFI_CUDA(cudaMemcpyAsync(o.data(), pr->out, o.size() * 4, cudaMemcpyDeviceToHost, pr->stream));
    if ((s = take_status(pr))) return s;
    for (int b = 0; b < batch; ++b)
        for (int j = 0; j < kOut; ++j) out_twists_host[b * kOut + j] = o[(size_t)b * kOutPad + j];
    return KIFI_OK;
}

kifi_status kifi_proposer_gradients(kifi_proposer* pr, const float* targets_dev, int batch, float* out_loss,
                                    float* out_grads_host) {
    if (!pr || !targets_dev) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    kifi_status s = check_batch(pr, batch);
    if (s) return s;
    KIFI_CUDA(cudaSetDevice(pr->device));
    if ((s = forward(pr, batch, true))) return s;
    KIFI_CUDA(cudaMemsetAsync(pr->loss, 0, 4, pr->stream));
    k_mse<<<blocks((size_t)batch * kOutPad), kThreads, 0, pr->stream>>>(pr->out, targets_dev, batch, pr->y2,
                                                                        pr->dbf, pr->loss);
    if ((s = backward(pr, batch))) return s;
    if (out_loss) KIFI_CUDA(cudaMemcpyAsync(out_loss, pr->loss, 4, cudaMemcpyDeviceToHost, pr->stream));
    if (out_grads_host)
        KIFI_CUDA(cudaMemcpyAsync(out_grads_host, pr->g, kLayout.total * 4, cudaMemcpyDeviceToHost, pr->stream));
    return take_status(pr);
}

kifi_status kifi_proposer_train_step(kifi_proposer* pr, const float* targets_dev, int batch, float lr,
                                     float* out_loss) {
    kifi_status s = kifi_proposer_gradients(pr, targets_dev, batch, out_loss, nullptr);
    if (s) return s;
    ++pr->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - (float)std::pow(b1, (double)pr->step), bc2 = 1.0f - (float)std::pow(b2, (double)pr->step);
    k_adam<<<blocks(kLayout.total), kThreads, 0, pr->stream>>>(pr->p, pr->g, pr->m1, pr->m2, pr->mask,
                                                              kLayout.total, lr, b1, b2, 1e-8f, bc1, bc2, pr->pb);
    KIFI_CUDA(cudaGetLastError());
    KIFI_CUDA(cudaStreamSynchronize(pr->stream));
    return KIFI_OK;
}

}  // extern "C"
