// kifi_icp.cu -- projective ICP on sm_103a: kifi::ICP::Align / AlignStep
// (KinectFission/kifi/ICP.cpp:9-265) and its target producers,
// Renderer::Bin (Renderer.cpp:39-80) and a depth back-projection.
//
// One AlignStep is two kernels, both ending in a last-CTA-done finisher, so a
// whole Align (any iteration count) is a fixed launch sequence with no host
// round trip:
//
//  k_icp_associate   one thread per source pixel of every row and every 4th
//                    column (ICP.cpp:66-67): back-project with the current
//                    pose estimate, project into the target camera, search
//                    the 21x21 window for the nearest valid target point
//                    within len^2 < 0.01 (:100-131; first minimum in scan
//                    order wins).  The pairs are stored; counts and the
//                    centroid sums are reduced with compensated float
//                    arithmetic per thread and warp (Kahan / TwoSum) and in
//                    double across CTAs.  The last CTA forms the centroids
//                    (:166-167).
//  k_icp_horn        the centred 3x3 cross-covariance (:169-197) with the
//                    same compensated reduction; the last CTA builds Horn's
//                    symmetric 4x4 matrix (:199-213) in double, finds its
//                    dominant eigenvector in double by Horn's closed form
//                    (characteristic quartic, Newton, adjugate; a cyclic
//                    Jacobi solve for degenerate spectra), turns it into
//                    R and t (:218-256) and accumulates the pose
//                    step * pose in double (:23-28).  The float pose the next
//                    association uses is that double pose rounded.
//
// The per-point arithmetic follows the reference's float expression order
// and x86 float-to-int conversion (CVTTSS2SI: truncation, INT_MIN for NaN or
// out-of-range); the reference's 640x480 window clamp (:108-109) is kept,
// with reads past the end of a smaller target buffer treated as invalid
// points.
#include "kifi_internal.h"

namespace kifi {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int cvt_i32_x86(float f) {
    if (f >= -2147483648.0f && f < 2147483648.0f) return __float2int_rz(f);
    return INT_MIN;
}
__device__ __forceinline__ int wrap_sub(int a, int b) { return (int)((unsigned int)a - (unsigned int)b); }

// Float-float (double-single) sums: a value is hi + lo with |lo| <= ulp(hi)/2.
// GB300 runs double precision at a small fraction of the float rate, so the
// compensated reductions stay in float pairs and only the final cross-CTA
// total is formed in double.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = fadd(a, b);
    float bb = fsub(s, a);
    e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = fadd(e, fadd(a.lo, b.lo));
    const float hi = fadd(s, e);
    return FF{hi, fsub(e, fsub(hi, s))};
}
__device__ __forceinline__ FF warp_sum_ff(FF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = ff_add(v, w);
    }
    return v;
}
__device__ __forceinline__ float load_depth(const void* depth, size_t i, bool u16) {
    if (u16) return fmul((float)(unsigned int)__ldg((const unsigned short*)depth + i), 0.001f);
    return __ldg((const float*)depth + i);
}

// last CTA to arrive returns true (after a fence); resets the counter
__device__ __forceinline__ bool last_cta(unsigned int* counter) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Totals of the per-CTA float-float partials of NV components, computed by
// the whole (last) CTA: thread t loads CTA t's partials (one round of
// independent loads), warps combine with float-float shuffles, and lane c of
// warp 0 adds the warp totals of component c in float-float and forms the
// double total.  Fixed order: independent of scheduling.  Double precision
// enters only at the end -- on GB300 a dependent double add costs about 64
// cycles against under 6 for a float one.
template <int NV>
__device__ __forceinline__ void moments_total(const IcpState* st, double* out) {
    __shared__ FF red[32][NV];
    FF a[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) a[c] = FF{0.0f, 0.0f};
    for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        float v[2 * NV];
#pragma unroll
        for (int c = 0; c < 2 * NV; ++c) v[c] = st->part[b * 48 + c];
#pragma unroll
        for (int c = 0; c < NV; ++c) a[c] = ff_add(a[c], FF{v[2 * c], v[2 * c + 1]});
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) a[c] = warp_sum_ff(a[c]);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) red[threadIdx.x >> 5][c] = a[c];
    __syncthreads();
    if (threadIdx.x < NV) {
        FF t = red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x / 32); ++w) t = ff_add(t, red[w][threadIdx.x]);
        out[threadIdx.x] = (double)t.hi + (double)t.lo;
    }
    __syncthreads();
}

constexpr int kTileCols = 8, kTileRows = 32;
constexpr int kStagePixels = 3840;  // float4 per pixel: 60 KB

// Scan of one thread's window in the staged region (float4 per pixel,
// `base` = its first candidate, odd row pitch).  Invalid target points were
// staged with x = NaN, which never passes `l2 < best`.  Three interleaved
// chains (columns mod 3) keep their own first strict minimum so that the
// compare/select dependencies overlap; the lexicographic (l2, candidate)
// minimum of the chains is the first strict minimum of the row-major scan.
// Returns the best squared distance (0.01 when none) and its candidate
// number r * 32 + c (-1 when none).
template <bool kW>
__device__ __forceinline__ float scan_staged(const float4* __restrict__ sp, int base, int pitch,
                                             int nr, int nc, float px, float py, float pz,
                                             float dw2, int* best_rc) {
    float b0 = 0.01f, b1 = 0.01f, b2 = 0.01f;
    int i0 = 0x7fffffff, i1 = 0x7fffffff, i2 = 0x7fffffff;
    auto cand = [&](int at, int rc, float& b, int& bi) {
        const float4 q = sp[at];
        const float dx = fsub(q.x, px), dy = fsub(q.y, py), dz = fsub(q.z, pz);
        const float zz = kW ? fadd(fmul(dz, dz), dw2) : fmul(dz, dz);
        const float l2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), zz);
        if (l2 < b) {
            b = l2;
            bi = rc;
        }
    };
    if (nc == 21) {
        for (int r = 0; r < nr; ++r, base += pitch) {
#pragma unroll
            for (int c = 0; c < 21; c += 3) {
                cand(base + c, r * 32 + c, b0, i0);
                cand(base + c + 1, r * 32 + c + 1, b1, i1);
                cand(base + c + 2, r * 32 + c + 2, b2, i2);
            }
        }
    } else {
        for (int r = 0; r < nr; ++r, base += pitch)
            for (int c = 0; c < nc; ++c) cand(base + c, r * 32 + c, b0, i0);
    }
    if (b1 < b0 || (b1 == b0 && i1 < i0)) {
        b0 = b1;
        i0 = i1;
    }
    if (b2 < b0 || (b2 == b0 && i2 < i0)) {
        b0 = b2;
        i0 = i2;
    }
    *best_rc = i0 == 0x7fffffff ? -1 : i0;
    return b0;
}

__device__ __noinline__ void finish_step(IcpState* __restrict__ st, const double* tot);

// One ICP::AlignStep (ICP.cpp:35-265) as one kernel.
//
// Association (:66-131): a CTA owns a tile of 8 source columns x 32 source
// rows.  Warp w takes source column w/2 of the tile and lane l source row l,
// so a warp's lanes are vertically adjacent sources whose windows sit about
// one image row apart; the two warps of a column split each 21x21 window
// into rows 0-10 and 11-20.  Each thread back-projects and projects its
// source, the CTA stages the bounding box of the tile's windows in shared
// memory (float4 per pixel, odd row pitch: lanes hit distinct banks) and each
// thread scans its rows in the reference's loop order; the halves are merged
// by (len^2, scan position), so the first strict minimum wins as in the
// reference.  A region too large for the staging buffer (fast motion) is
// read from global memory instead.  Target pixel (y1, x1) is linear index
// y1 * synth_w + x1 as in the reference; indices past the buffer's end are
// invalid points.
//
// Horn's sums: instead of a second pass over the pairs for the centred
// cross-covariance (:169-197), the kernel accumulates the raw moments --
// count, sum p, sum q, sum p_r q_c (each product split exactly into a
// float-float pair by an FMA) and the squared distances -- in float-float
// per warp and CTA; the last CTA to finish totals them in double, forms the
// centroids and S = sum p q^T - n mu_p mu_q^T in double, and runs the Horn
// solve.  Algebraically this is the reference's two-pass sum; numerically it
// is at least as accurate.
constexpr int kAssocThreads = 512;
constexpr int kMoments = 17;  // n, p xyz, q xyz, p q^T (9), len^2

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = fmul(a, b);
    return FF{p, __fmaf_rn(a, b, -p)};  // exact remainder of the product
}

__global__ void __launch_bounds__(kAssocThreads, 2) k_icp_step(IcpArgs a, IcpState* __restrict__ st) {
    extern __shared__ float4 stage[];  // kStagePixels target points
    __shared__ int s_box[4];
    __shared__ float s_hb[kTileCols][32];  // lower half's best len^2 per source
    __shared__ int s_hi[kTileCols][32];    // and its candidate number
    __shared__ FF s_acc[kTileCols][kMoments];
    const int n_cols = (a.width + 3) / 4;
    const int tiles_x = (n_cols + kTileCols - 1) / kTileCols;
    const int tiles_y = (a.height + kTileRows - 1) / kTileRows;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wcol = warp >> 1, half = warp & 1;
    const float half_w = fmul((float)a.synth_w, 0.5f), half_h = fmul((float)a.synth_h, 0.5f);
    const size_t n_synth = (size_t)a.synth_w * a.synth_h;
    if (half == 0 && lane < kMoments) s_acc[wcol][lane] = FF{0.0f, 0.0f};
    if (threadIdx.x == 0) atomicMin(&st->t_start, global_ns());
    for (int tile = blockIdx.x; tile < tiles_x * tiles_y; tile += gridDim.x) {
        const int tx = tile % tiles_x, ty = tile / tiles_x;
        const int col = tx * kTileCols + wcol, y = ty * kTileRows + lane;
        const bool mine = col < n_cols && y < a.height;
        float wp[4] = {0.f, 0.f, 0.f, 0.f};
        int u = 0, v = 0, nr = 0, nc = 0;
        if (mine) {
            const int x = col * 4;
            const float d = load_depth(a.depth, (size_t)y * a.width + x, a.depth_u16);
            if (0.0f != d) {
                float pt[4], cl[4];
                pt[0] = fmul(fadd(fmul((float)x, a.fl_inv_x), a.pp_x), d);
                pt[1] = fmul(fadd(fmul(-(float)y, a.fl_inv_y), a.pp_y), d);
                pt[2] = fmul(fadd(fmul(-1.0f, 1.0f), 0.0f), d);
                pt[3] = 1.0f;
                mat_vec(st->pose_f, pt, wp);
                mat_vec(a.proj, wp, cl);
                const float ux = fdiv(cl[0], cl[3]), uy = fdiv(cl[1], cl[3]);
                u = wrap_sub(cvt_i32_x86(fadd(fmul(ux, half_w), half_w)), 10);
                v = wrap_sub(wrap_sub(a.synth_h - 1, cvt_i32_x86(fadd(fmul(uy, half_h), half_h))), 10);
                u = max(0, u);
                v = max(0, v);
                nr = (int)min(480ll, (long long)v + 21) - v;
                nc = (int)min(640ll, (long long)u + 21) - u;
                if (nr <= 0 || nc <= 0) nr = nc = 0;
            }
        }
        // bounding box of the tile's windows
        if (threadIdx.x == 0) {
            s_box[0] = 0x7fffffff; s_box[1] = 0x7fffffff; s_box[2] = -1; s_box[3] = -1;
        }
        __syncthreads();
        if (half == 0) {  // warp-uniform; one shared atomic per warp and bound
            const bool has = nr > 0;
            const int mu0 = (int)__reduce_min_sync(0xffffffffu, has ? (unsigned)u : 0x7fffffffu);
            const int mv0 = (int)__reduce_min_sync(0xffffffffu, has ? (unsigned)v : 0x7fffffffu);
            const int mu1 = __reduce_max_sync(0xffffffffu, has ? u + nc : -1);
            const int mv1 = __reduce_max_sync(0xffffffffu, has ? v + nr : -1);
            if (lane == 0 && mu1 >= 0) {
                atomicMin(&s_box[0], mu0);
                atomicMin(&s_box[1], mv0);
                atomicMax(&s_box[2], mu1);
                atomicMax(&s_box[3], mv1);
            }
        }
        __syncthreads();
        const int bx0 = s_box[0], by0 = s_box[1], bx1 = s_box[2], by1 = s_box[3];
        const int bw = bx1 - bx0, bh = by1 - by0;
        const int pitch = bw | 1;  // odd pitch: vertically adjacent windows hit distinct banks
        const bool staged = bx1 >= 0 && pitch * bh <= kStagePixels;
        if (staged) {
            for (int i = threadIdx.x; i < bw * bh; i += kAssocThreads) {
                const int ry = i / bw, rx = i - ry * bw;
                const size_t at = (size_t)(by0 + ry) * a.synth_w + (bx0 + rx);
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                if (at < n_synth) q = __ldg(a.synth + at);
                // (0,0,0) = no point (ICP.cpp:112): stage it as NaN
                if (q.x == 0.0f && q.y == 0.0f && q.z == 0.0f) q.x = __int_as_float(0x7fffffff);
                stage[ry * pitch + rx] = q;
            }
        }
        __syncthreads();
        // this thread's rows of the window
        const int r0 = half ? 11 : 0, r1 = half ? nr : min(nr, 11);
        float best = 0.01f;
        int rc = -1;
        float3 bq = make_float3(0.f, 0.f, 0.f);
        if (r1 > r0) {
            const float dw = fsub(1.0f, wp[3]);
            const float dw2 = fmul(dw, dw);
            if (staged) {
                const int base = (v + r0 - by0) * pitch + (u - bx0);
                // dz^2 + dw^2 == dz^2 exactly when dw == 0 (dz^2 >= 0)
                best = dw2 != 0.0f
                           ? scan_staged<true>(stage, base, pitch, r1 - r0, nc, wp[0], wp[1], wp[2], dw2, &rc)
                           : scan_staged<false>(stage, base, pitch, r1 - r0, nc, wp[0], wp[1], wp[2], dw2, &rc);
                if (rc >= 0) {
                    const float4 q = stage[base + (rc >> 5) * pitch + (rc & 31)];
                    bq = make_float3(q.x, q.y, q.z);
                    rc += r0 * 32;
                }
            } else {
                for (int r = r0; r < r1; ++r) {
                    for (int c = 0; c < nc; ++c) {
                        const size_t at = (size_t)(v + r) * a.synth_w + (u + c);
                        if (at >= n_synth) continue;
                        const float4 q = __ldg(a.synth + at);
                        if (q.x == 0.0f && q.y == 0.0f && q.z == 0.0f) continue;
                        const float dx = fsub(q.x, wp[0]), dy = fsub(q.y, wp[1]), dz = fsub(q.z, wp[2]);
                        const float l2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fadd(fmul(dz, dz), dw2));
                        if (l2 < best) {
                            best = l2;
                            rc = r * 32 + c;
                            bq = make_float3(q.x, q.y, q.z);
                        }
                    }
                }
            }
        }
        // merge the halves: the upper rows come earlier in scan order
        if (half == 1) {
            s_hb[wcol][lane] = best;
            s_hi[wcol][lane] = rc;
        }
        __syncthreads();
        if (half == 0) {
            const float ob = s_hb[wcol][lane];
            const int oi = s_hi[wcol][lane];
            if (oi >= 0 && (rc < 0 || ob < best)) {
                best = ob;
                rc = oi;
                const size_t at = (size_t)(v + (oi >> 5)) * a.synth_w + (u + (oi & 31));
                const float4 q = staged ? stage[(v + (oi >> 5) - by0) * pitch + (u + (oi & 31) - bx0)]
                                        : __ldg(a.synth + at);
                bq = make_float3(q.x, q.y, q.z);
            }
            const bool hit = mine && rc >= 0;
            // this tile's raw moments, folded into the warp's accumulators
            if (__any_sync(0xffffffffu, hit)) {
                const float px = hit ? wp[0] : 0.f, py = hit ? wp[1] : 0.f, pz = hit ? wp[2] : 0.f;
                const float qx = hit ? bq.x : 0.f, qy = hit ? bq.y : 0.f, qz = hit ? bq.z : 0.f;
                const float pv[3] = {px, py, pz}, qv[3] = {qx, qy, qz};
#pragma unroll
                for (int i = 0; i < kMoments; ++i) {
                    FF m;
                    if (i == 0) m = FF{hit ? 1.0f : 0.0f, 0.0f};
                    else if (i < 4) m = FF{pv[i - 1], 0.0f};
                    else if (i < 7) m = FF{qv[i - 4], 0.0f};
                    else if (i < 16) m = two_prod(pv[(i - 7) / 3], qv[(i - 7) % 3]);
                    else m = FF{hit ? best : 0.0f, 0.0f};
                    const FF w = warp_sum_ff(m);
                    if (lane == 0) s_acc[wcol][i] = ff_add(s_acc[wcol][i], w);
                }
            }
        }
        __syncthreads();  // staging buffer and half results are reused by the next tile
    }
    if (threadIdx.x < kMoments) {
        FF t = s_acc[0][threadIdx.x];
        for (int w = 1; w < kTileCols; ++w) t = ff_add(t, s_acc[w][threadIdx.x]);
        st->part[blockIdx.x * 48 + 2 * threadIdx.x] = t.hi;
        st->part[blockIdx.x * 48 + 2 * threadIdx.x + 1] = t.lo;
        __threadfence();  // publish before the CTA signals completion
    }
    if (threadIdx.x == 0) atomicMax(&st->t_body, global_ns());
    if (!last_cta(&st->done)) return;
    __shared__ double tot[kMoments];
    moments_total<kMoments>(st, tot);
    if (threadIdx.x < 32) finish_step(st, tot);
}

// ------------------------------------------------------ FP64 Horn solve
// Cyclic Jacobi on a symmetric 4x4 (row-major) in double; V accumulates the
// rotations (columns are eigenvectors).  Starting from V0 (the previous
// solve's eigenvectors) the matrix is first rotated into that basis.
__device__ __noinline__ void jacobi4(double* A, double* V, const double* V0, bool warm) {
    double a[16];
    if (warm) {
        double t[16];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                double s = 0.0;
                for (int k = 0; k < 4; ++k) s += A[4 * i + k] * V0[4 * k + j];
                t[4 * i + j] = s;
            }
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                double s = 0.0;
                for (int k = 0; k < 4; ++k) s += V0[4 * k + i] * t[4 * k + j];
                a[4 * i + j] = s;
            }
        for (int i = 0; i < 16; ++i) V[i] = V0[i];
    } else {
        for (int i = 0; i < 16; ++i) {
            a[i] = A[i];
            V[i] = (i % 5 == 0) ? 1.0 : 0.0;
        }
    }
    double scale = 0.0;
    for (int i = 0; i < 16; ++i) scale += a[i] * a[i];
    // converged once the off-diagonal mass is below (1e-13)^2 of the total:
    // tighter bounds sit at double rounding noise and never terminate early
    for (int sweep = 0; sweep < 32; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) off += a[4 * p + q] * a[4 * p + q];
        if (!(off > 1e-26 * scale)) break;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 4; ++q) {
                const double apq = a[4 * p + q];
                if (apq == 0.0) continue;
                const double theta = (a[4 * q + q] - a[4 * p + p]) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 4; ++k) {
                    const double akp = a[4 * k + p], akq = a[4 * k + q];
                    a[4 * k + p] = c * akp - s * akq;
                    a[4 * k + q] = s * akp + c * akq;
                }
                for (int k = 0; k < 4; ++k) {
                    const double apk = a[4 * p + k], aqk = a[4 * q + k];
                    a[4 * p + k] = c * apk - s * aqk;
                    a[4 * q + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 4; ++k) {
                    const double vkp = V[4 * k + p], vkq = V[4 * k + q];
                    V[4 * k + p] = c * vkp - s * vkq;
                    V[4 * k + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 4; ++i) A[i] = a[5 * i];  // eigenvalues into A[0..3]
}

// Warp 0 of the last CTA of an AlignStep: totals of the raw moments, the
// centroids and the centred cross-covariance S (ICP.cpp:166-197), Horn's
// symmetric N (:199-213), its dominant eigenvector, R and t (:215-256) and
// pose <- (T R) pose (:23-28) -- all in double.
//
// GB300 executes double precision at a small fraction of the float rate, and
// this tail runs on one SM while the others wait, so it is written for a
// short dependent chain: every quantity with independent entries gets a lane
// of its own, sums are shuffle trees, and divisions / square roots start from
// a float approximation refined by Newton steps in double.
//
// The eigenvector is Horn's closed form (B. K. P. Horn, "Closed-form solution
// of absolute orientation using unit quaternions", JOSA A 4(4), 1987): the
// characteristic polynomial det(lambda I - N) from the Faddeev-LeVerrier
// recursion, its largest root by Newton's method started from an upper bound
// of the spectrum (Gershgorin, or the Frobenius norm; right of its largest
// root the polynomial is increasing and convex, so the iterates fall
// monotonically onto the root), and the largest column of adj(N - lambda I),
// which is proportional to the eigenvector when the root is simple.  A
// repeated largest root falls back to the cyclic Jacobi solver.
__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}
__device__ __forceinline__ double recip_d(double x) {  // 1/x to double accuracy
    double r = (double)(1.0f / (float)x);
    r = r * (2.0 - x * r);
    return r * (2.0 - x * r);
}
__device__ __forceinline__ double rsqrt_d(double x) {  // 1/sqrt(x) to double accuracy
    double y = (double)rsqrtf((float)x);
    y = y * (1.5 - 0.5 * x * y * y);
    return y * (1.5 - 0.5 * x * y * y);
}

__device__ __noinline__ void finish_step(IcpState* __restrict__ st, const double* tot) {
    __shared__ double sN[16], sM[16], sA[16], sT[16], sq[4];
    __shared__ int s_ok;
    const int lane = threadIdx.x;
    const double n = tot[0];
    const double inv_n = recip_d(n);
    // S_rc = sum p_r q_c - n mu_r nu_c, lane j < 9 holds S_j
    const int jr = lane < 9 ? lane / 3 : 0, jc = lane < 9 ? lane % 3 : 0;
    double mu[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) mu[i] = tot[1 + i] * inv_n;
    const double pq = tot[7 + (lane < 9 ? lane : 0)];
    const double Sj = pq - n * mu[jr] * mu[3 + jc];
    double S[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) S[i] = __shfl_sync(0xffffffffu, Sj, i);
    const double Sxx = S[0], Sxy = S[1], Sxz = S[2], Syx = S[3], Syy = S[4], Syz = S[5],
                 Szx = S[6], Szy = S[7], Szz = S[8];
    if (lane < 16) {
        const double N[16] = {Sxx + Syy + Szz, Syz - Szy, Szx - Sxz, Sxy - Syx,
                              Syz - Szy, Sxx - Syy - Szz, Sxy + Syx, Szx + Sxz,
                              Szx - Sxz, Sxy + Syx, Syy - Sxx - Szz, Syz + Szy,
                              Sxy - Syx, Szx + Sxz, Syz + Szy, Szz - Sxx - Syy};
        double v = N[0];
#pragma unroll
        for (int i = 1; i < 16; ++i)
            if (lane == i) v = N[i];
        sN[lane] = sM[lane] = v;
    }
    __syncwarp();
    const int r = (lane >> 2) & 3, c = lane & 3;
    // upper bounds of the spectrum: Frobenius norm and Gershgorin rows
    const double fro2 = warp_sum_d(lane < 16 ? sN[lane] * sN[lane] : 0.0);
    const double fro = (double)sqrtf((float)fro2) * (1.0 + 1e-6);
    double gr = lane < 4 ? sN[5 * lane] : -1e300;
    if (lane < 4)
        for (int j = 0; j < 4; ++j)
            if (j != lane) gr += fabs(sN[4 * lane + j]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gr = fmax(gr, __shfl_xor_sync(0xffffffffu, gr, o));
    // Faddeev-LeVerrier: p(l) = l^4 + c3 l^3 + c2 l^2 + c1 l + c0
    auto trace4 = [&](double mine) {  // sum of the diagonal lanes 0, 5, 10, 15
        double t = (lane < 16 && r == c) ? mine : 0.0;
        return warp_sum_d(t);
    };
    double cf[4];
    cf[3] = -trace4(lane < 16 ? sM[lane] : 0.0);
    for (int k = 2; k <= 4; ++k) {
        const double ck = cf[5 - k];
        double t = 0.0;
        if (lane < 16)
            for (int j = 0; j < 4; ++j) t += sN[4 * r + j] * (sM[4 * j + c] + (j == c ? ck : 0.0));
        __syncwarp();
        if (lane < 16) sM[lane] = t;
        __syncwarp();
        cf[4 - k] = -trace4(t) * (k == 2 ? 0.5 : (k == 3 ? (1.0 / 3.0) : 0.25));
    }
    double l = fmin(fro, gr);
    for (int it = 0; it < 60; ++it) {
        const double p = (((l + cf[3]) * l + cf[2]) * l + cf[1]) * l + cf[0];
        const double dp = ((4.0 * l + 3.0 * cf[3]) * l + 2.0 * cf[2]) * l + cf[1];
        if (!(dp > 0.0)) break;
        const double step = p * recip_d(dp);
        l -= step;
        if (!(fabs(step) > 1e-15 * fro)) break;
    }
    if (lane < 16) sA[lane] = sN[lane] - (r == c ? l : 0.0);
    __syncwarp();
    auto cof = [&](int row, int col) {  // (row, col) cofactor of A
        int rr[3], cc[3], nn = 0, m = 0;
        for (int i = 0; i < 4; ++i)
            if (i != row) rr[nn++] = i;
        for (int j = 0; j < 4; ++j)
            if (j != col) cc[m++] = j;
        const double d =
            sA[4 * rr[0] + cc[0]] * (sA[4 * rr[1] + cc[1]] * sA[4 * rr[2] + cc[2]] - sA[4 * rr[1] + cc[2]] * sA[4 * rr[2] + cc[1]]) -
            sA[4 * rr[0] + cc[1]] * (sA[4 * rr[1] + cc[0]] * sA[4 * rr[2] + cc[2]] - sA[4 * rr[1] + cc[2]] * sA[4 * rr[2] + cc[0]]) +
            sA[4 * rr[0] + cc[2]] * (sA[4 * rr[1] + cc[0]] * sA[4 * rr[2] + cc[1]] - sA[4 * rr[1] + cc[1]] * sA[4 * rr[2] + cc[0]]);
        return ((row + col) & 1) ? -d : d;
    };
    double dj = lane < 4 ? fabs(cof(lane, lane)) : -1.0;
    int bj = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xffffffffu, dj, o);
        const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (od > dj || (od == dj && oj < bj)) {
            dj = od;
            bj = oj;
        }
    }
    const bool ok = dj > 1e-24 * fro * fro * fro;
    const double qk = (ok && lane < 4) ? cof(lane, bj) : 0.0;
    const double inv_norm = rsqrt_d(warp_sum_d(qk * qk));
    if (lane < 4) sq[lane] = qk * inv_norm;
    if (lane == 0) s_ok = ok;
    __syncwarp();
    if (!s_ok && lane == 0) {
        double A[16], V[16];
        for (int i = 0; i < 16; ++i) A[i] = sN[i];
        jacobi4(A, V, V, false);
        int imax = 0;
        for (int i = 1; i < 4; ++i)
            if (A[i] > A[imax]) imax = i;
        double nn = 0.0;
        for (int i = 0; i < 4; ++i) nn += V[4 * i + imax] * V[4 * i + imax];
        nn = sqrt(nn);
        for (int i = 0; i < 4; ++i) sq[i] = V[4 * i + imax] / nn;
    }
    __syncwarp();
    // R from the quaternion (x = scalar part, ICP.cpp:233-254), one entry per lane
    const double qx = sq[0], qy = sq[1], qz = sq[2], qw = sq[3];
    double Rj = 0.0;
    switch (lane) {
        case 0: Rj = 1.0 - 2.0 * (qz * qz + qw * qw); break;
        case 1: Rj = 2.0 * (qy * qz - qx * qw); break;
        case 2: Rj = 2.0 * (qy * qw + qx * qz); break;
        case 3: Rj = 2.0 * (qy * qz + qx * qw); break;
        case 4: Rj = 1.0 - 2.0 * (qy * qy + qw * qw); break;
        case 5: Rj = 2.0 * (qz * qw - qx * qy); break;
        case 6: Rj = 2.0 * (qy * qw - qx * qz); break;
        case 7: Rj = 2.0 * (qz * qw + qx * qy); break;
        case 8: Rj = 1.0 - 2.0 * (qy * qy + qz * qz); break;
        default: break;
    }
    double R[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = __shfl_sync(0xffffffffu, Rj, i);
    // step = T * R with t = mu_q - R mu_p (row-major 4x4), one entry per lane
    if (lane < 16) {
        double v;
        if (r == 3) v = (c == 3) ? 1.0 : 0.0;
        else if (c < 3) v = R[3 * r + c];
        else v = mu[3 + r] - (R[3 * r] * mu[0] + R[3 * r + 1] * mu[1] + R[3 * r + 2] * mu[2]);
        sT[lane] = v;
    }
    __syncwarp();
    double pnew = 0.0;
    if (lane < 16)
        for (int k = 0; k < 4; ++k) pnew += sT[4 * r + k] * st->pose[4 * k + c];
    __syncwarp();
    if (lane < 16) {
        st->pose[lane] = pnew;
        st->pose_f[4 * c + r] = (float)pnew;
    }
    if (lane == 0) {
        st->n_assoc = (int)(n + 0.5);
        st->sum_l2 = tot[16];
        for (int i = 0; i < 3; ++i) {
            st->mu_s[i] = (float)mu[i];
            st->mu_d[i] = (float)mu[3 + i];
        }
        const int it = st->iter;
        if (it < kIcpMaxStats) {
            st->stats[it].n_assoc = (int)(n + 0.5);
            st->stats[it].rms = n > 0.0 ? (double)sqrtf((float)(tot[16] * inv_n)) : 0.0;
            const unsigned long long t_end = global_ns();
            st->stats[it].body_us = (float)(st->t_body - st->t_start) * 1e-3f;
            st->stats[it].tail_us = (float)(t_end - st->t_body) * 1e-3f;
        }
        st->t_start = ~0ull;
        st->t_body = 0ull;
        st->iter = it + 1;
    }
}

__global__ void k_icp_begin(IcpState* st, Mat4 guess) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) st->pose[4 * r + c] = (double)guess.m[4 * c + r];
    for (int i = 0; i < 16; ++i) st->pose_f[i] = guess.m[i];
    st->iter = 0;
    st->have_V = 0;
    st->done = 0u;
    st->t_start = ~0ull;
    st->t_body = 0ull;
}

// World points of a depth frame: the back-projection of
// DepthMap2PointCloud (Integrator.cpp:121-144) without the voxel step;
// pixels without depth get (0,0,0), the reference's "invalid" target value.
__global__ void k_backproject(const void* __restrict__ depth, int u16, int width, int height,
                              float fl_inv_x, float fl_inv_y, float pp_x, float pp_y, Mat4 e2w,
                              float4* __restrict__ out) {
    const int n = width * height;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int v = i / width, u = i - v * width;
        const float d = load_depth(depth, i, u16 != 0);
        float w[4] = {0.f, 0.f, 0.f, 0.f};
        if (d > 0.0f) {
            float p[4];
            p[0] = fadd(fmul(fadd(fmul((float)u, fl_inv_x), pp_x), d), 0.0f);
            p[1] = fadd(fmul(fadd(fmul(fadd(0.0f, -(float)v), fl_inv_y), pp_y), d), 0.0f);
            p[2] = fadd(fmul(fadd(fmul(-1.0f, 1.0f), 0.0f), d), 0.0f);
            p[3] = fadd(fmul(fadd(fmul(0.0f, 1.0f), 0.0f), d), 1.0f);
            mat_vec(e2w.m, p, w);
        }
        out[i] = make_float4(w[0], w[1], w[2], 0.0f);
    }
}

// host float3 target -> the float4 layout the association reads (one
// 16-byte load per candidate)
__global__ void k_expand_target(const float* __restrict__ in, int n, float4* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.0f);
}

// Renderer::Bin: a z-buffered splat.  The first point (in input order) with
// the smallest clip-space z wins a pixel, as the reference's sequential
// strict "<" test does; a 64-bit atomicMin over (ordered z, point index)
// gives the same winner in parallel.
__device__ __forceinline__ unsigned int ordered_bits(float z) {
    if (z == 0.0f) z = 0.0f;  // -0 and +0 compare equal
    unsigned int b = __float_as_uint(z);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void k_bin_splat(const float* __restrict__ pts, unsigned int n, Mat4 w2c, int width,
                            int height, unsigned long long* __restrict__ zbuf) {
    const float hw = fmul((float)width, 0.5f), hh = fmul((float)height, 0.5f);
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float p[4] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], 1.0f}, c[4];
        mat_vec(w2c.m, p, c);
        const float x = fdiv(c[0], c[3]), y = fdiv(c[1], c[3]), z = fdiv(c[2], c[3]);
        const int u = cvt_i32_x86(fadd(fmul(x, hw), hw));
        const int v = wrap_sub(height - 1, cvt_i32_x86(fadd(fmul(y, hh), hh)));
        if (u >= 0 && u < width && v >= 0 && v < height && z >= -1.0f && z <= 1.0f)
            atomicMin(zbuf + (size_t)v * width + u, (unsigned long long)ordered_bits(z) << 32 | i);
    }
}

__global__ void k_bin_resolve(const float* __restrict__ pts, const unsigned long long* __restrict__ zbuf,
                              int n_pix, float* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pix; i += gridDim.x * blockDim.x) {
        const unsigned long long z = zbuf[i];
        float x = 0.f, y = 0.f, w = 0.f;
        if (z != ~0ull) {
            const unsigned int j = (unsigned int)(z & 0xffffffffu);
            x = pts[3 * j];
            y = pts[3 * j + 1];
            w = pts[3 * j + 2];
        }
        out[3 * i] = x;
        out[3 * i + 1] = y;
        out[3 * i + 2] = w;
    }
}

}  // namespace

cudaError_t icp_align_enqueue(const IcpArgs& a, IcpState* st, const Mat4& guess, int iterations,
                              int /*ctas*/, cudaStream_t stream) {
    k_icp_begin<<<1, 32, 0, stream>>>(st, guess);
    const int n_cols = (a.width + 3) / 4;
    const int tiles = ((n_cols + kTileCols - 1) / kTileCols) * ((a.height + kTileRows - 1) / kTileRows);
    const int ctas = tiles < kIcpMaxCtas ? tiles : kIcpMaxCtas;
    const size_t smem = kStagePixels * sizeof(float4);
    cudaError_t e =
        cudaFuncSetAttribute(k_icp_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    for (int it = 0; it < iterations; ++it) k_icp_step<<<ctas, kAssocThreads, smem, stream>>>(a, st);
    return cudaGetLastError();
}

cudaError_t expand_target_enqueue(const float* in, int n, float4* out, int ctas, cudaStream_t st) {
    k_expand_target<<<ctas, kThreads, 0, st>>>(in, n, out);
    return cudaGetLastError();
}

cudaError_t backproject_enqueue(const void* depth, bool u16, const kifi_camera& cam,
                                const Mat4& eye_to_world, float4* out, int ctas, cudaStream_t st) {
    const float fix = fdiv(1.0f, cam.fx), fiy = fdiv(1.0f, cam.fy);
    const float ppx = fmul(fsub(0.5f, cam.cx), fix), ppy = fmul(fsub(cam.cy, 0.5f), fiy);
    k_backproject<<<ctas, kThreads, 0, st>>>(depth, u16 ? 1 : 0, cam.width, cam.height, fix, fiy,
                                             ppx, ppy, eye_to_world, out);
    return cudaGetLastError();
}

cudaError_t bin_enqueue(const float* pts, unsigned int n, const Mat4& w2c, int width, int height,
                        unsigned long long* zbuf, float* out, int ctas, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(zbuf, 0xff, (size_t)width * height * 8, st);
    if (e) return e;
    if (n) k_bin_splat<<<ctas, kThreads, 0, st>>>(pts, n, w2c, width, height, zbuf);
    k_bin_resolve<<<ctas, kThreads, 0, st>>>(pts, zbuf, width * height, out);
    return cudaGetLastError();
}

}  // namespace kifi
