// kifi_icp.cu -- projective ICP on sm_103a: kifi::ICP::Align / AlignStep
// (KinectFission/kifi/ICP.cpp:9-265) and its target producers,
// Renderer::Bin (Renderer.cpp:39-80) and a depth back-projection.
//
// One AlignStep is one kernel, k_icp_step, ending in a last-CTA-done
// finisher, so a whole Align (any iteration count) is a fixed launch sequence
// with no host round trip:
//
//  association   every row and every 4th column (ICP.cpp:66-67) is a source
//                pixel: back-project it with the current pose estimate,
//                project into the target camera, search the 21x21 window for
//                the nearest valid target point within len^2 < 0.01
//                (:100-131; the first minimum in scan order wins).  CTAs own
//                tiles of sources and stage the union of their windows in
//                shared memory.
//  moments       the associated pairs are not stored: count, sum p, sum q,
//                sum p q^T and the squared distances are accumulated per
//                CTA in float-float, each product split exactly by an FMA.
//  finisher      the last CTA totals the per-CTA partials, and one warp
//                forms the centroids and the centred cross-covariance
//                (:166-197), Horn's matrix (:199-213), its dominant
//                eigenvector (:215-231), R and t (:233-261) and the pose
//                update (:20-28), without double precision (see the Horn
//                solve below).
//
// Consecutive steps are programmatic dependent launches: the next step's
// grid is scheduled once every CTA has finished its association, and waits
// (griddepcontrol.wait) for the finisher before it reads the pose.
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

// Float-float (double-single) arithmetic: a value is hi + lo with |lo| about
// ulp(hi)/2 or less -- a 48-bit significand.  GB300 issues double precision
// at a small fraction of the float rate, so every compensated sum and the
// Horn solve's precise steps use float pairs instead.
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
__device__ __forceinline__ FF ff_norm(float hi, float lo) {  // |lo| may exceed ulp(hi)/2
    const float s = fadd(hi, lo);
    return FF{s, fsub(lo, fsub(s, hi))};
}
__device__ __forceinline__ FF operator+(FF a, FF b) { return ff_add(a, b); }
__device__ __forceinline__ FF operator-(FF a, FF b) { return ff_add(a, FF{-b.hi, -b.lo}); }
__device__ __forceinline__ FF operator-(FF a) { return FF{-a.hi, -a.lo}; }
__device__ __forceinline__ FF operator*(FF a, FF b) {
    const float p = fmul(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
    return ff_norm(p, e);
}
__device__ __forceinline__ FF operator*(FF a, float b) {
    const float p = fmul(a.hi, b);
    return ff_norm(p, __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p)));
}
__device__ __forceinline__ FF ff_div(FF a, FF b) {  // a / b, b != 0
    const float q1 = fdiv(a.hi, b.hi);
    const FF r = a - b * q1;
    return ff_norm(q1, fdiv(r.hi, b.hi));
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

// Last CTA to arrive returns true and gets the grid's total of `mine` (an
// association count, read after the barrier); resets the counter.  The
// counter holds finished CTAs in its high 32 bits and the running total in
// its low 32 bits, so one atomic does both.  Thread 0's atomic orders the
// whole CTA's earlier stores (the barrier makes them visible to it) before
// the count, and the count before the last CTA's reads.
__device__ __forceinline__ bool last_cta(unsigned long long* counter, const unsigned int& mine,
                                         unsigned int* total, unsigned int nblk) {
    __shared__ bool last;
    __shared__ unsigned int s_total;
    __syncthreads();
    if (threadIdx.x == 0) {
        // one acquire-release atomic at gpu scope: the release (cumulative
        // over the CTA's writes ordered before it by the barrier) publishes
        // this CTA's partials; the acquire lets the last CTA read everyone's
        const unsigned long long add = (1ull << 32) | mine;
        unsigned long long prev;
        asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;"
                     : "=l"(prev) : "l"(counter), "l"(add) : "memory");
        last = (unsigned int)(prev >> 32) == nblk - 1;
        s_total = (unsigned int)prev + mine;
        if (last) *counter = 0ull;  // read again only by the next launch
    }
    __syncthreads();
    *total = s_total;
    return last;
}

// Totals of the per-CTA float-float partials, by the whole (last) CTA.  The
// partials are stored component-major (hi row, then lo row, each
// kIcpMaxCtas long), so warp w reduces component w + 1 (the count, component
// 0, comes with the last-CTA counter) with coalesced loads: lane l adds CTAs
// l, l + 32, ... in float-float -- all of a lane's loads (up to 320 CTAs)
// issued in one round -- then a shuffle tree.
// Fixed order: independent of scheduling.  The loads bypass L1 (the partials
// were written by other SMs during this launch).
constexpr int kTotalsPerLane = 10;
__device__ __forceinline__ FF lane_partials(const float* ph, int b0, int G) {
    float h[kTotalsPerLane], l[kTotalsPerLane];
#pragma unroll
    for (int k = 0; k < kTotalsPerLane; ++k) {
        const int b = b0 + 32 * k;
        h[k] = b < G ? __ldcg(ph + b) : 0.0f;
        l[k] = b < G ? __ldcg(ph + kIcpMaxCtas + b) : 0.0f;
    }
    FF acc{h[0], l[0]};
#pragma unroll
    for (int k = 1; k < kTotalsPerLane; ++k) acc = ff_add(acc, FF{h[k], l[k]});
    return acc;
}
template <int NV>
__device__ __forceinline__ void moments_total(const IcpState* st, unsigned int count, FF* out, int G) {
    const int lane = threadIdx.x & 31, c = (threadIdx.x >> 5) + 1;
    if (threadIdx.x == 0) out[0] = FF{(float)count, 0.0f};  // exact: at most 2^24 sources
    if (c < NV) {
        FF a{0.0f, 0.0f};
        for (int b0 = lane; b0 < G; b0 += 32 * kTotalsPerLane)
            a = ff_add(a, lane_partials(st->part + (size_t)(2 * c) * kIcpMaxCtas, b0, G));
        a = warp_sum_ff(a);
        if (lane == 0) out[c] = a;
    }
    __syncthreads();
}

constexpr int kTileCols = 8, kTileRows = 32;
constexpr int kSplitRow = 10;   // window rows [0, 10) to the lower half-warp set, [10, 21) to the upper
constexpr int kStageBatch = 4;  // staging loads in flight per thread
constexpr int kStagePixels = 5120;  // three float planes (x, y, z): 60 KB
constexpr int kPredMargin = 2;      // pixels added around a predicted window box

// Row pitch of a staged region `w` pixels wide: even, so that a pair of
// adjacent pixels is one aligned 64-bit load, with pitch/2 odd, so that the
// 64-bit loads of lanes whose windows sit one row apart hit distinct banks.
__host__ __device__ constexpr int stage_pitch(int w) {
    return ((w + 1) & ~1) + ((((w + 1) & ~1) >> 1) & 1 ? 0 : 2);
}

// Packed float pairs (f32x2): each half is rounded exactly as the scalar
// __fsub_rn / __fadd_rn of that half.  Products are formed as
// fma(a, a, -0) with the -0 a kernel parameter: that is the rounded product
// for every input (x + -0 = x, also for x = -0), and unlike a packed
// multiply it cannot be fused into the add that consumes it -- ptxas does
// fuse mul.rn.f32x2 into a following add.rn.f32x2, which would round the
// sum of squares once instead of the reference's separate roundings.
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
    unsigned long long d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_sq(unsigned long long a, unsigned long long neg_zero) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(d) : "l"(a), "l"(neg_zero));
    return d;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// The staging buffer: planes of x, y and z, kStagePixels floats each.
struct Stage {
    float* x;
    float* y;
    float* z;
};

// The target pixels [x0, x0 + w) x [y0, y0 + h) (linear index y * synth_w + x,
// as the reference reads them) into the planes of `stage` with row pitch
// `pitch`, by the whole CTA: kStageBatch independent loads in flight per
// thread, then the stores.  (0,0,0) is no point (ICP.cpp:112) and is staged
// with x = NaN; indices past the buffer's end are invalid points too.
__device__ __forceinline__ void stage_region(const Stage& stage, const float4* __restrict__ synth,
                                             size_t n_synth, int synth_w, int x0, int y0, int w, int h,
                                             int pitch) {
    // warps take rows (kStageBatch rows in flight each), lanes take columns
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, n_warps = blockDim.x >> 5;
    for (int ry0 = warp; ry0 < h; ry0 += kStageBatch * n_warps) {
        for (int rx = lane; rx < w; rx += 32) {
            float4 q[kStageBatch];
#pragma unroll
            for (int k = 0; k < kStageBatch; ++k) {
                const int ry = ry0 + k * n_warps;
                q[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (ry < h) {
                    const size_t at = (size_t)(y0 + ry) * synth_w + (x0 + rx);
                    if (at < n_synth) q[k] = __ldg(synth + at);
                }
            }
#pragma unroll
            for (int k = 0; k < kStageBatch; ++k) {
                const int ry = ry0 + k * n_warps;
                if (ry < h) {
                    if (q[k].x == 0.0f && q[k].y == 0.0f && q[k].z == 0.0f) q[k].x = __int_as_float(0x7fffffff);
                    const int at = ry * pitch + rx;
                    stage.x[at] = q[k].x;
                    stage.y[at] = q[k].y;
                    stage.z[at] = q[k].z;
                }
            }
        }
    }
}

// Scan of one thread's window in the staged region (`base` = its first
// candidate's plane index, even pitch).  Invalid target points were staged
// with x = NaN, which never passes `l2 < best`.  A full 21-wide row is ten
// aligned pairs of adjacent candidates, whose squared distances are formed
// two at a time in packed float pairs (each half with the reference's
// operations and rounding), plus the one candidate left over: the first when
// the window starts on an odd plane index, else the last.  Three chains --
// the pairs' first halves, their second halves and the leftovers -- keep
// their own first strict minimum; the lexicographic (l2, candidate) minimum
// of the chains is the first strict minimum of the row-major scan.  Returns
// the best squared distance (0.01 when none) and its candidate number
// r * 32 + c (-1 when none).
template <bool kW>
__device__ __forceinline__ float scan_staged(const Stage& sp, int base, int pitch, int nr, int nc, float px,
                                             float py, float pz, float dw2, float neg_zero, int* best_rc) {
    float b0 = 0.01f, b1 = 0.01f, b2 = 0.01f;
    int i0 = 0x7fffffff, i1 = 0x7fffffff, i2 = 0x7fffffff;
    // one candidate in scalar float, the reference's order: (dx^2 + dy^2) + (dz^2 + dw^2)
    auto cand = [&](int at, int c, float& b, int& bc) {
        const float dx = fsub(sp.x[at], px), dy = fsub(sp.y[at], py), dz = fsub(sp.z[at], pz);
        const float zz = kW ? fadd(fmul(dz, dz), dw2) : fmul(dz, dz);
        const float l2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), zz);
        if (l2 < b) {
            b = l2;
            bc = c;
        }
    };
    if (nc == 21) {
        const int o = base & 1;       // the pairs start at an even plane index
        const int cs = o ? 0 : 20;    // the leftover candidate's column
        const unsigned long long PX = f2_pack(px, px), PY = f2_pack(py, py), PZ = f2_pack(pz, pz);
        const unsigned long long DW = f2_pack(dw2, dw2), NZ = f2_pack(neg_zero, neg_zero);
        for (int r = 0; r < nr; ++r, base += pitch) {
            // a candidate records only its pair number (a constant of the
            // unrolled row); the row and the parity are folded in once per row
            int c0 = -1, c1 = -1;
            bool moved = false;
            const int pb = base + o;
#pragma unroll
            for (int k = 0; k < 10; ++k) {
                const int at = pb + 2 * k;
                const unsigned long long X = *(const unsigned long long*)(sp.x + at);
                const unsigned long long Y = *(const unsigned long long*)(sp.y + at);
                const unsigned long long Z = *(const unsigned long long*)(sp.z + at);
                const unsigned long long dx = f2_sub(X, PX), dy = f2_sub(Y, PY), dz = f2_sub(Z, PZ);
                unsigned long long zz = f2_sq(dz, NZ);
                if (kW) zz = f2_add(zz, DW);
                const unsigned long long l2 = f2_add(f2_add(f2_sq(dx, NZ), f2_sq(dy, NZ)), zz);
                float lo, hi;
                f2_unpack(l2, lo, hi);
                if (lo < b0) {
                    b0 = lo;
                    c0 = 2 * k;
                }
                if (hi < b1) {
                    b1 = hi;
                    c1 = 2 * k;
                }
            }
            {
                int cl = -1;
                cand(base + cs, 0, b2, cl);
                moved = cl >= 0;
            }
            const int r32 = r * 32;
            if (c0 >= 0) i0 = r32 + o + c0;
            if (c1 >= 0) i1 = r32 + o + c1 + 1;
            if (moved) i2 = r32 + cs;
        }
    } else {
        for (int r = 0; r < nr; ++r, base += pitch) {
            int c0 = -1;
            for (int c = 0; c < nc; ++c) cand(base + c, c, b0, c0);
            if (c0 >= 0) i0 = r * 32 + c0;
        }
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

__device__ __noinline__ void finish_step(IcpState* __restrict__ st, const FF* __restrict__ tot,
                                        IcpPoseMail* mail, unsigned long long mail_seq);

// One ICP::AlignStep (ICP.cpp:35-265) as one kernel.
//
// Association (:66-131): a CTA owns a tile of 8 source columns x 32 source
// rows.  Warp w takes source column w/2 of the tile and lane l source row l,
// so a warp's lanes are vertically adjacent sources whose windows sit about
// one image row apart; the two warps of a column split each 21x21 window
// into rows 0-10 and 11-20.  Each thread back-projects and projects its
// source, the CTA stages the bounding box of the tile's windows in shared
// memory (planes of x, y and z; an even row pitch with pitch/2 odd: pairs of
// pixels are aligned 64-bit loads, lanes hit distinct banks) and each
// thread scans its rows in the reference's loop order, two candidates at a
// time in packed float pairs; the halves are merged
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
// per warp and CTA; the last CTA to finish totals them, forms the centroids
// and S = sum p q^T - (sum p) mu_q^T in float-float, and runs the Horn
// solve.  Algebraically this is the reference's two-pass sum; numerically it
// is more accurate than the reference's float Kahan sums.
constexpr int kAssocThreads = 512;
constexpr int kMoments = 17;  // n, p xyz, q xyz, p q^T (9), len^2
static_assert(kAssocThreads / 32 == kMoments - 1, "one warp per moment after the count");

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = fmul(a, b);
    return FF{p, __fmaf_rn(a, b, -p)};  // exact remainder of the product
}

// One AlignStep of one frame pair; `blk` / `nblk`: this CTA's index among
// the nblk CTAs that work on the pair (the launch's own grid, or a share of
// a batched launch over several pairs).
__device__ __forceinline__ void icp_step_body(const IcpArgs& a, IcpState* __restrict__ st, unsigned int blk,
                                              unsigned int nblk) {
    extern __shared__ float4 stage_mem[];  // three planes of kStagePixels floats
    const Stage stage{(float*)stage_mem, (float*)stage_mem + kStagePixels, (float*)stage_mem + 2 * kStagePixels};
    __shared__ int s_box[4];
    __shared__ float s_hb[kTileCols][32];  // lower half's best len^2 per source
    __shared__ int s_hi[kTileCols][32];    // and its candidate number
    __shared__ FF s_acc[kMoments];             // this CTA's moments (index 0 unused: s_count)
    __shared__ float s_rec[7][kTileCols * 32];  // per source: p xyz, q xyz, len^2 (0 when no pair)
    __shared__ unsigned int s_count;
    // Steps are launched programmatically behind one another: this grid may
    // start while the previous step's last CTA still updates the pose.  Wait
    // for that grid (and its memory) before touching the ICP state.
    const int n_cols = (a.width + 3) / 4;
    const int tiles_x = (n_cols + kTileCols - 1) / kTileCols;
    const int tiles_y = (a.height + kTileRows - 1) / kTileRows;
    const size_t n_synth = (size_t)a.synth_w * a.synth_h;
    // While the previous step may still be finishing: stage the box this
    // CTA's first tile covered then, plus a margin -- windows move little
    // between steps.  The box is read by one thread (it may be stale or
    // half-updated; any box is only a guess) and shared, so every thread
    // stages the same region; after the wait the guess is used only if it
    // holds every window.
    __shared__ int s_pred[4];
    if (threadIdx.x == 0) {
        int p[4] = {0, 0, 0, 0};
        if (blk < tiles_x * tiles_y) {
            const volatile int* tb = st->tile_box + 4 * blk;
            const int b0 = tb[0], b1 = tb[1], b2 = tb[2], b3 = tb[3];
            if (b2 > b0 && b3 > b1 && b0 >= 0 && b1 >= 0) {
                const int x0 = max(b0 - kPredMargin, 0), y0 = max(b1 - kPredMargin, 0);
                const int w = b2 + kPredMargin - x0, h = b3 + kPredMargin - y0;
                if (w <= kStagePixels && h <= kStagePixels && stage_pitch(w) * h <= kStagePixels) {
                    p[0] = x0;
                    p[1] = y0;
                    p[2] = w;
                    p[3] = h;
                }
            }
        }
        s_pred[0] = p[0];
        s_pred[1] = p[1];
        s_pred[2] = p[2];
        s_pred[3] = p[3];
    }
    __syncthreads();
    const int px0 = s_pred[0], py0 = s_pred[1], pw = s_pred[2], ph = s_pred[3];
    if (pw > 0) stage_region(stage, a.synth, n_synth, a.synth_w, px0, py0, pw, ph, stage_pitch(pw));
    // this thread's source of the first tile in eye space (no pose needed yet)
    const int lane0 = threadIdx.x & 31, wcol0 = (threadIdx.x >> 5) >> 1;
    float pre_d = 0.0f;
    {
        const int t0 = blk;
        if (t0 < tiles_x * tiles_y) {
            const int col = (t0 % tiles_x) * kTileCols + wcol0, y = (t0 / tiles_x) * kTileRows + lane0;
            if (col < n_cols && y < a.height) pre_d = load_depth(a.depth, (size_t)y * a.width + col * 4, a.depth_u16);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wcol = warp >> 1, half = warp & 1;
    const float half_w = fmul((float)a.synth_w, 0.5f), half_h = fmul((float)a.synth_h, 0.5f);
    if (threadIdx.x < kMoments) s_acc[threadIdx.x] = FF{0.0f, 0.0f};
    if (threadIdx.x == 0) s_count = 0u;
    if (threadIdx.x == 0) atomicMin(&st->t_start, global_ns());
    for (int tile = blk; tile < tiles_x * tiles_y; tile += nblk) {
        const int tx = tile % tiles_x, ty = tile / tiles_x;
        const int col = tx * kTileCols + wcol, y = ty * kTileRows + lane;
        const bool mine = col < n_cols && y < a.height;
        float wp[4] = {0.f, 0.f, 0.f, 0.f};
        int u = 0, v = 0, nr = 0, nc = 0;
        if (mine) {
            const int x = col * 4;
            const float d = tile == (int)blk ? pre_d : load_depth(a.depth, (size_t)y * a.width + x, a.depth_u16);
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
        const int ax0 = s_box[0], ay0 = s_box[1], ax1 = s_box[2], ay1 = s_box[3];
        // the prefetched region if it holds every window of the tile, else stage the box now
        const bool use_pred = tile == (int)blk && pw > 0 && ax1 >= 0 && ax0 >= px0 && ay0 >= py0 &&
                              ax1 <= px0 + pw && ay1 <= py0 + ph;
        int bx0 = ax0, by0 = ay0, pitch = stage_pitch(ax1 - ax0);
        bool staged;
        if (use_pred) {
            bx0 = px0;
            by0 = py0;
            pitch = stage_pitch(pw);
            staged = true;
        } else {
            staged = ax1 >= 0 && pitch * (ay1 - ay0) <= kStagePixels;
            if (staged) stage_region(stage, a.synth, n_synth, a.synth_w, ax0, ay0, ax1 - ax0, ay1 - ay0, pitch);
        }
        if (threadIdx.x == 0 && tile < kIcpMaxCtas && ax1 >= 0) {
            int* tb = st->tile_box + 4 * tile;
            tb[0] = ax0;
            tb[1] = ay0;
            tb[2] = ax1;
            tb[3] = ay1;
        }
        __syncthreads();
        // this thread's rows of the window
        const int r0 = half ? kSplitRow : 0, r1 = half ? nr : min(nr, kSplitRow);
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
                           ? scan_staged<true>(stage, base, pitch, r1 - r0, nc, wp[0], wp[1], wp[2], dw2,
                                               a.neg_zero, &rc)
                           : scan_staged<false>(stage, base, pitch, r1 - r0, nc, wp[0], wp[1], wp[2], dw2,
                                                a.neg_zero, &rc);
                if (rc >= 0) {
                    const int at = base + (rc >> 5) * pitch + (rc & 31);
                    bq = make_float3(stage.x[at], stage.y[at], stage.z[at]);
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
                if (staged) {
                    const int at = (v + (oi >> 5) - by0) * pitch + (u + (oi & 31) - bx0);
                    bq = make_float3(stage.x[at], stage.y[at], stage.z[at]);
                } else {
                    const float4 q = __ldg(a.synth + (size_t)(v + (oi >> 5)) * a.synth_w + (u + (oi & 31)));
                    bq = make_float3(q.x, q.y, q.z);
                }
            }
            const bool hit = mine && rc >= 0;
            if (a.pairs && mine) {
                const size_t k = (size_t)y * n_cols + col;
                a.pairs[k] = hit ? (long long)(v + (rc >> 5)) * a.synth_w + (u + (rc & 31)) : -1ll;
                a.pairs_len2[k] = hit ? best : 0.01f;
            }
            // this source's pair for the tile's moments (zeros when none)
            const int sidx = wcol * 32 + lane;
            s_rec[0][sidx] = hit ? wp[0] : 0.f;
            s_rec[1][sidx] = hit ? wp[1] : 0.f;
            s_rec[2][sidx] = hit ? wp[2] : 0.f;
            s_rec[3][sidx] = hit ? bq.x : 0.f;
            s_rec[4][sidx] = hit ? bq.y : 0.f;
            s_rec[5][sidx] = hit ? bq.z : 0.f;
            s_rec[6][sidx] = hit ? best : 0.f;
            const unsigned int nh = __popc(__ballot_sync(0xffffffffu, hit));
            if (lane == 0 && nh) atomicAdd(&s_count, nh);
        }
        __syncthreads();
        // the tile's raw moments: warp w reduces moment w + 1 over the 256
        // sources (lane l takes sources l, l + 32, ...), in float-float
        {
            const int c = warp + 1;
            FF acc{0.0f, 0.0f};
#pragma unroll
            for (int k = 0; k < kTileCols; ++k) {
                const int sidx = lane + 32 * k;
                FF m;
                if (c < 7) m = FF{s_rec[c - 1][sidx], 0.0f};
                else if (c < 16) m = two_prod(s_rec[(c - 7) / 3][sidx], s_rec[3 + (c - 7) % 3][sidx]);
                else m = FF{s_rec[6][sidx], 0.0f};
                acc = ff_add(acc, m);
            }
            acc = warp_sum_ff(acc);
            if (lane == 0) s_acc[c] = ff_add(s_acc[c], acc);
        }
        __syncthreads();  // staging buffer, half results and records are reused by the next tile
    }
    // association done: the next step's grid may be scheduled (it waits above)
    asm volatile("griddepcontrol.launch_dependents;");
    if (threadIdx.x >= 1 && threadIdx.x < kMoments) {
        const FF t = s_acc[threadIdx.x];
        st->part[(size_t)(2 * threadIdx.x) * kIcpMaxCtas + blk] = t.hi;
        st->part[(size_t)(2 * threadIdx.x + 1) * kIcpMaxCtas + blk] = t.lo;
    }
    if (threadIdx.x == 0) atomicMax(&st->t_body, global_ns());
    unsigned int n_total;
    if (!last_cta(&st->done, s_count, &n_total, nblk)) return;
    __shared__ FF tot[kMoments];
    moments_total<kMoments>(st, n_total, tot, (int)nblk);
    if (threadIdx.x < 32) finish_step(st, tot, a.mail, a.mail_seq);
}

__global__ void __launch_bounds__(kAssocThreads, 2) k_icp_step(IcpArgs a, IcpState* __restrict__ st) {
    icp_step_body(a, st, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------- Horn solve
// Cyclic Jacobi on a symmetric 4x4 (row-major) in double; V accumulates the
// rotations (columns are eigenvectors), the eigenvalues end in A[0..3].  The
// fallback for spectra whose largest eigenvalue is (nearly) repeated.
__device__ __noinline__ void jacobi4(double* A, double* V) {
    double a[16];
    for (int i = 0; i < 16; ++i) {
        a[i] = A[i];
        V[i] = (i % 5 == 0) ? 1.0 : 0.0;
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
    for (int i = 0; i < 4; ++i) A[i] = a[5 * i];
}

// Horn's closed form (B. K. P. Horn, "Closed-form solution of absolute
// orientation using unit quaternions", JOSA A 4(4), 1987), written for one
// thread and without double precision: GB300 issues a double instruction
// (conversions included) at about one per 64 cycles per SM sub-partition,
// even for a single thread, and this tail runs on one SM while the others
// wait.  Precision comes from float-float (FF) arithmetic where it matters.
//
//  1. FF: centroids, the centred cross-covariance S = sum p q^T - (sum p)
//     mu_q^T (the raw moments cancel heavily) and Horn's symmetric N, scaled
//     by a power of two to unit size (exact).
//  2. float: the characteristic polynomial of N by the Faddeev-LeVerrier
//     recursion, its largest root by Newton's method from an upper bound of
//     the spectrum (Gershgorin or the Frobenius norm; right of the largest
//     root the polynomial is increasing and convex, so the iterates fall
//     monotonically onto it), and the largest diagonal entry j of
//     adj(N - lambda I), whose column j is then proportional to the
//     eigenvector.
//  3. FF: one step of Rayleigh-quotient inverse iteration -- rho = q'Nq / q'q,
//     q <- column j of adj(N - rho I) -- which converges cubically, so the
//     float-accurate start lands well below float rounding (two steps when
//     the eigen-gaps are small).
//  4. A spectrum whose gap product (the adjugate diagonal above) is tiny --
//     a nearly repeated largest eigenvalue -- goes to the double Jacobi
//     solver instead.
//
// R, t and the accumulated pose are FF as well; the float pose the next
// association uses is the FF pose rounded (its high part).
//
// Symmetric 4x4 matrices are held as their upper triangle, row by row.
__host__ __device__ constexpr int sym(int i, int j) {
    return i <= j ? (i * (7 - i)) / 2 + j : (j * (7 - j)) / 2 + i;
}
template <typename T>
__device__ __forceinline__ T shifted(const T* n, T s, int i, int j) {
    return i == j ? n[sym(i, i)] - s : n[sym(i, j)];
}
// determinant of rows r0..r2 and columns k0..k2 of N - s I
template <typename T>
__device__ __forceinline__ T minor3(const T* n, T s, int r0, int r1, int r2, int k0, int k1, int k2) {
    const T a00 = shifted(n, s, r0, k0), a01 = shifted(n, s, r0, k1), a02 = shifted(n, s, r0, k2);
    const T a10 = shifted(n, s, r1, k0), a11 = shifted(n, s, r1, k1), a12 = shifted(n, s, r1, k2);
    const T a20 = shifted(n, s, r2, k0), a21 = shifted(n, s, r2, k1), a22 = shifted(n, s, r2, k2);
    return a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
}
// column j of adj(N - s I) (the matrix is symmetric, so cofactor (i, j))
template <typename T>
__device__ __forceinline__ void adj_column(const T* n, T s, int j, T* q) {
    switch (j) {
        case 0:
            q[0] = minor3(n, s, 1, 2, 3, 1, 2, 3);
            q[1] = -minor3(n, s, 1, 2, 3, 0, 2, 3);
            q[2] = minor3(n, s, 1, 2, 3, 0, 1, 3);
            q[3] = -minor3(n, s, 1, 2, 3, 0, 1, 2);
            break;
        case 1:
            q[0] = -minor3(n, s, 0, 2, 3, 1, 2, 3);
            q[1] = minor3(n, s, 0, 2, 3, 0, 2, 3);
            q[2] = -minor3(n, s, 0, 2, 3, 0, 1, 3);
            q[3] = minor3(n, s, 0, 2, 3, 0, 1, 2);
            break;
        case 2:
            q[0] = minor3(n, s, 0, 1, 3, 1, 2, 3);
            q[1] = -minor3(n, s, 0, 1, 3, 0, 2, 3);
            q[2] = minor3(n, s, 0, 1, 3, 0, 1, 3);
            q[3] = -minor3(n, s, 0, 1, 3, 0, 1, 2);
            break;
        default:
            q[0] = -minor3(n, s, 0, 1, 2, 1, 2, 3);
            q[1] = minor3(n, s, 0, 1, 2, 0, 2, 3);
            q[2] = -minor3(n, s, 0, 1, 2, 0, 1, 3);
            q[3] = minor3(n, s, 0, 1, 2, 0, 1, 2);
            break;
    }
}
// out = n (p + c I); symmetric because p is a polynomial in n
__device__ __forceinline__ void sym_mul_shift(const float* n, const float* p, float c, float* out) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i; j < 4; ++j) {
            float t = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) t = fmaf(n[sym(i, k)], k == j ? p[sym(k, j)] + c : p[sym(k, j)], t);
            out[sym(i, j)] = t;
        }
}

// Warp 0 of the last CTA of an AlignStep: from the totals of the raw
// moments, the centroids and S (ICP.cpp:166-197), N (:199-213), its dominant
// eigenvector (above), R and t (:215-256) and pose <- (T R) pose (:20-28).
// The work is spread over the lanes entry by entry -- centroids, S, N,
// the four minors and cofactors, R, t and the twelve pose entries -- and
// joined by shuffles; the float characteristic polynomial and its Newton
// search run on every lane alike.  Symmetric matrices indexed by a lane go
// through shared memory (a register array indexed by a lane would live in
// local memory).
__device__ __forceinline__ FF shfl_ff(FF v, int src) {
    return FF{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}
// minor3 of rows {0..3} \ {rx} and columns {0..3} \ {cx} of n - s I, n in
// shared memory (upper triangle), for lane-dependent rx, cx
template <typename T>
__device__ __forceinline__ T minor_excl(const T* n, T s, int rx, int cx) {
    const int r0 = rx == 0 ? 1 : 0, r1 = rx <= 1 ? 2 : 1, r2 = rx <= 2 ? 3 : 2;
    const int k0 = cx == 0 ? 1 : 0, k1 = cx <= 1 ? 2 : 1, k2 = cx <= 2 ? 3 : 2;
    return minor3(n, s, r0, r1, r2, k0, k1, k2);
}
// N's entry k (upper triangle, row by row) as (S[i1] s2 S[i2]) s3 S[i3]:
// N = [[Sxx+Syy+Szz, Syz-Szy, Szx-Sxz, Sxy-Syx], [., Sxx-Syy-Szz, Sxy+Syx,
// Szx+Sxz], [., ., Syy-Sxx-Szz, Syz+Szy], [., ., ., Szz-Sxx-Syy]] (:199-213)
__device__ __forceinline__ void n_terms(int k, int& i1, int& i2, int& i3, bool& m2, bool& m3, bool& t3) {
    // per k (4 bits each): i1, i2, i3; flags: minus second, minus third, has third
    constexpr unsigned long long kI1 = 0x8546101650ull, kI2 = 0x0702343274ull, kI3 = 0x4080080008ull;
    constexpr unsigned int kM2 = 0x29e, kM3 = 0x290, kT3 = 0x291;
    i1 = (int)(kI1 >> (4 * k)) & 15;
    i2 = (int)(kI2 >> (4 * k)) & 15;
    i3 = (int)(kI3 >> (4 * k)) & 15;
    m2 = (kM2 >> k) & 1u;
    m3 = (kM3 >> k) & 1u;
    t3 = (kT3 >> k) & 1u;
}

__device__ __noinline__ void finish_step(IcpState* __restrict__ st, const FF* __restrict__ tot,
                                        IcpPoseMail* mail, unsigned long long mail_seq) {
    __shared__ float s_f[10];
    __shared__ FF s_nf[10];
    const int lane = threadIdx.x & 31;
    // the step's counters for the statistics, read now so that no load is
    // left behind the pose update (final: every CTA wrote them before its
    // release of the last-CTA counter)
    int step = 0;
    unsigned long long t_start = 0ull, t_body = 0ull;
    if (lane == 0) {
        step = __ldcg(&st->iter);
        t_start = __ldcg(&st->t_start);
        t_body = __ldcg(&st->t_body);
    }
    // 1. centroids (lanes 0-5), S (lanes 0-8), N (lanes 0-9) in FF
    const float n = fadd(tot[0].hi, tot[0].lo);  // an exact count below 2^24
    FF my_mu{0.0f, 0.0f};
    if (lane < 6) {
        const float h = fdiv(tot[1 + lane].hi, n);
        const float r = fadd(__fmaf_rn(-h, n, tot[1 + lane].hi), tot[1 + lane].lo);  // exact remainder + lo
        my_mu = ff_norm(h, fdiv(r, n));
    }
    const int sl = lane < 9 ? lane : 0;
    const FF mu_c = shfl_ff(my_mu, 3 + sl % 3);
    const FF my_s = tot[7 + sl] - tot[1 + sl / 3] * mu_c;
    int i1, i2, i3;
    bool m2, m3, t3;
    n_terms(lane < 10 ? lane : 0, i1, i2, i3, m2, m3, t3);
    const FF a1 = shfl_ff(my_s, i1), a2 = shfl_ff(my_s, i2), a3 = shfl_ff(my_s, i3);
    FF my_n = m2 ? a1 - a2 : a1 + a2;
    if (t3) my_n = m3 ? my_n - a3 : my_n + a3;
    const bool diag = lane == 0 || lane == 4 || lane == 7 || lane == 9;
    float f2 = lane < 10 ? fmul(diag ? my_n.hi : 2.0f * my_n.hi, my_n.hi) : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) f2 = fadd(f2, __shfl_xor_sync(0xffffffffu, f2, o));
    // power-of-two scale 2^-e/2 with f2 = m 2^e: N's Frobenius norm lands in [0.5, 1.5)
    const int e = ((__float_as_int(f2) >> 23) & 0xff) - 127;
    const float sc = __int_as_float((127 - (e >> 1)) << 23);
    const bool finite = f2 > 1e-30f && f2 < 1e30f;
    if (lane < 10) {
        s_nf[lane] = FF{my_n.hi * sc, my_n.lo * sc};
        s_f[lane] = my_n.hi * sc;
    }
    __syncwarp();
    float f[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) f[i] = s_f[i];
    // 2. float search (every lane)
    float gmax = -1e30f;  // Gershgorin: the largest row bound
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float t = f[sym(i, i)];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j != i) t += fabsf(f[sym(i, j)]);
        gmax = fmaxf(gmax, t);
    }
    // start just above the smaller of the Gershgorin and Frobenius bounds
    float l = fminf(gmax, sqrtf(f2 * sc * sc)) * 1.00001f + 1e-6f;
    float m[10], w[10];
    const float c3 = -(f[0] + f[4] + f[7] + f[9]);
    sym_mul_shift(f, f, c3, m);
    const float c2 = -0.5f * (m[0] + m[4] + m[7] + m[9]);
    sym_mul_shift(f, m, c2, w);
    const float c1 = -(w[0] + w[4] + w[7] + w[9]) * (1.0f / 3.0f);
    float tr = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) tr = fmaf(f[sym(i, k)], k == i ? w[sym(k, i)] + c1 : w[sym(k, i)], tr);
    const float c0 = -0.25f * tr;
    for (int it = 0; it < 32; ++it) {
        const float p = fmaf(fmaf(fmaf(l + c3, l, c2), l, c1), l, c0);
        const float dp = fmaf(fmaf(fmaf(4.0f, l, 3.0f * c3), l, 2.0f * c2), l, c1);
        if (!(dp > 0.0f)) break;
        const float step = __fdividef(p, dp);
        if (!(step > 0.0f)) break;
        l -= step;
        if (step <= 1e-7f * fabsf(l)) break;
    }
    // the principal minors (lanes 0-3); j = the first largest
    const int q4 = lane & 3;
    const float my_d = fabsf(minor_excl(s_f, l, q4, q4));
    int j = 0;
    float dj = __shfl_sync(0xffffffffu, my_d, 0);
#pragma unroll
    for (int i = 1; i < 4; ++i) {
        const float di = __shfl_sync(0xffffffffu, my_d, i);
        if (di > dj) {
            j = i;
            dj = di;
        }
    }
    // cofactor (i, j) of a symmetric matrix: lane i takes q[i] = (-1)^(i+j) minor(rows != j, cols != i)
    const bool neg = ((q4 + j) & 1) != 0;
    FF my_q{0.0f, 0.0f};
    int solver = 0;
    if (finite && dj > 1e-4f) {
        // 3. Rayleigh-quotient inverse iteration in FF
        float my_qf = minor_excl(s_f, l, j, q4);
        if (neg) my_qf = -my_qf;
        const int steps = dj < 1e-2f ? 2 : 1;
        for (int s = 0; s < steps; ++s) {
            // lane r: row r of N times qf, then the Rayleigh quotient num / qq over lanes 0-3
            FF t{0.0f, 0.0f};
#pragma unroll
            for (int c = 0; c < 4; ++c) t = t + s_nf[sym(q4, c)] * __shfl_sync(0xffffffffu, my_qf, c);
            FF num = lane < 4 ? t * my_qf : FF{0.0f, 0.0f};
            FF qq = lane < 4 ? FF{my_qf, 0.0f} * my_qf : FF{0.0f, 0.0f};
#pragma unroll
            for (int o = 1; o < 4; o <<= 1) {
                num = num + shfl_ff(num, lane ^ o);
                qq = qq + shfl_ff(qq, lane ^ o);
            }
            num = shfl_ff(num, 0);
            qq = shfl_ff(qq, 0);
            my_q = minor_excl(s_nf, ff_div(num, qq), j, q4);
            if (neg) my_q = -my_q;
            my_qf = my_q.hi;
        }
    } else {
        // 4. nearly repeated largest eigenvalue (or no finite solution)
        solver = 1;
        if (lane == 0) {
            double A[16], V[16];
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) A[4 * r + c] = (double)s_nf[sym(r, c)].hi + (double)s_nf[sym(r, c)].lo;
            jacobi4(A, V);
            int imax = 0;
            for (int i = 1; i < 4; ++i)
                if (A[i] > A[imax]) imax = i;
            for (int i = 0; i < 4; ++i) {
                const double vi = V[4 * i + imax];
                s_nf[i] = FF{(float)vi, (float)(vi - (double)(float)vi)};  // N is not needed any more
            }
        }
        __syncwarp();
        my_q = s_nf[q4];
    }
    // q = normalize(q) (:231): 1/sqrt(q'q) from a float estimate and one FF Newton step
    FF qq = lane < 4 ? my_q * my_q : FF{0.0f, 0.0f};
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) qq = qq + shfl_ff(qq, lane ^ o);
    qq = shfl_ff(qq, 0);
    const float r0 = rsqrtf(qq.hi);
    const FF corr = (FF{1.0f, 0.0f} - qq * r0 * r0) * (0.5f * r0);
    my_q = my_q * (FF{r0, 0.0f} + corr);
    // R from the quaternion, x = scalar part (:233-254), in FF: lane k < 9 takes entry k
    //   diagonal k = 0, 4, 8:  1 - 2 (q_a q_a + q_b q_b)
    //   off-diagonal:          2 (q_a q_b +- q_c q_d)
    const int rk = lane < 9 ? lane : 0;
    // (a, b, c, d) per entry, 4 bits each: (2,2,3,3) (1,2,0,3) (1,3,0,2) (1,2,0,3) (1,1,3,3)
    // (2,3,0,1) (1,3,0,2) (2,3,0,1) (1,1,2,2)
    constexpr unsigned long long kA = 0x121211112ull, kB = 0x133312322ull, kC = 0x200030003ull,
                                 kD = 0x212133233ull;
    const int ia = (int)(kA >> (4 * rk)) & 15, ib = (int)(kB >> (4 * rk)) & 15;
    const int ic = (int)(kC >> (4 * rk)) & 15, id = (int)(kD >> (4 * rk)) & 15;
    const FF qa = shfl_ff(my_q, ia), qb = shfl_ff(my_q, ib), qc = shfl_ff(my_q, ic), qd = shfl_ff(my_q, id);
    const FF pab = qa * qb, pcd = qc * qd;
    const bool rdiag = rk == 0 || rk == 4 || rk == 8;
    const bool rminus = rk == 1 || rk == 5 || rk == 6;
    const FF my_r = rdiag ? FF{1.0f, 0.0f} - (pab + pcd) * 2.0f : (rminus ? pab - pcd : pab + pcd) * 2.0f;
    // t = dstMedian - R srcMedian (:256): lane r < 3
    const int tr3 = lane < 3 ? lane : 0;
    const FF mu0 = shfl_ff(my_mu, 0), mu1 = shfl_ff(my_mu, 1), mu2 = shfl_ff(my_mu, 2);
    const FF mud = shfl_ff(my_mu, 3 + tr3);
    const FF my_t = mud - (shfl_ff(my_r, 3 * tr3) * mu0 + shfl_ff(my_r, 3 * tr3 + 1) * mu1 +
                           shfl_ff(my_r, 3 * tr3 + 2) * mu2);
    // pose <- [R t; 0 1] pose (:259-263, :20-28): lane k < 12 takes row r = k % 3 of column c = k / 3
    const int pk = lane < 12 ? lane : 0, pc = pk / 3, pr = pk - 3 * pc;
    FF P[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) P[i] = FF{st->pose_f[4 * pc + i], st->pose_lo[4 * pc + i]};
    const FF v = shfl_ff(my_r, 3 * pr) * P[0] + shfl_ff(my_r, 3 * pr + 1) * P[1] + shfl_ff(my_r, 3 * pr + 2) * P[2] +
                 shfl_ff(my_t, pr) * P[3];
    __syncwarp();  // every lane has read its column before any entry is replaced
    if (lane < 12) {
        st->pose_f[4 * pc + pr] = v.hi;
        st->pose_lo[4 * pc + pr] = v.lo;
    }
    const FF md0 = shfl_ff(my_mu, 3), md1 = shfl_ff(my_mu, 4), md2 = shfl_ff(my_mu, 5);
    // the alignment's last step publishes the pose to the host's mailbox (a
    // launch argument, null in the other steps): lanes 0-11 their new entries,
    // lanes 0, 3, 6, 9 their column's unchanged bottom entry, then lane 0 the number
    if (mail) {
        if (lane < 12) {
            mail->pose[4 * pc + pr] = v.hi;
            if (pr == 0) mail->pose[4 * pc + 3] = P[3].hi;
        }
        __threadfence_system();
        __syncwarp();
        if (lane == 0) *(volatile unsigned long long*)&mail->seq = mail_seq;
    }
    if (lane != 0) return;
    st->n_assoc = (int)n;
    st->mu_s[0] = fadd(mu0.hi, mu0.lo);
    st->mu_s[1] = fadd(mu1.hi, mu1.lo);
    st->mu_s[2] = fadd(mu2.hi, mu2.lo);
    st->mu_d[0] = fadd(md0.hi, md0.lo);
    st->mu_d[1] = fadd(md1.hi, md1.lo);
    st->mu_d[2] = fadd(md2.hi, md2.lo);
    if (step < kIcpMaxStats) {
        st->stats[step].n_assoc = (int)n;
        st->stats[step].solver = solver;
        st->stats[step].sum_l2 = fadd(tot[16].hi, tot[16].lo);
        const unsigned long long t_end = global_ns();
        // spans below 2^32 ns: the 32-bit conversions round as the 64-bit ones
        st->stats[step].body_us = (float)(unsigned int)(t_body - t_start) * 1e-3f;
        st->stats[step].tail_us = (float)(unsigned int)(t_end - t_body) * 1e-3f;
    }
    st->t_start = ~0ull;
    st->t_body = 0ull;
    st->iter = step + 1;
}

__device__ __forceinline__ void icp_begin_body(IcpState* st, const Mat4& guess) {
    for (int i = 0; i < 16; ++i) {
        st->pose_f[i] = guess.m[i];
        st->pose_lo[i] = 0.0f;
    }
    st->iter = 0;
    st->done = 0ull;
    st->t_start = ~0ull;
    st->t_body = 0ull;
}

__global__ void k_icp_begin(IcpState* st, Mat4 guess) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    icp_begin_body(st, guess);
}

// World points of a depth frame: the back-projection of
// DepthMap2PointCloud (Integrator.cpp:121-144) without the voxel step;
// pixels without depth get (0,0,0), the reference's "invalid" target value.
__device__ __forceinline__ void backproject_body(const void* __restrict__ depth, int u16, int width, int height,
                                                 float fl_inv_x, float fl_inv_y, float pp_x, float pp_y,
                                                 const Mat4& e2w, float4* __restrict__ out, unsigned int blk,
                                                 unsigned int nblk) {
    const int n = width * height;
    for (int i = blk * blockDim.x + threadIdx.x; i < n; i += nblk * blockDim.x) {
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

__global__ void k_backproject(const void* __restrict__ depth, int u16, int width, int height,
                              float fl_inv_x, float fl_inv_y, float pp_x, float pp_y, Mat4 e2w,
                              float4* __restrict__ out) {
    backproject_body(depth, u16, width, height, fl_inv_x, fl_inv_y, pp_x, pp_y, e2w, out, blockIdx.x, gridDim.x);
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

// ---- batched: several frame pairs per launch, each pair's CTAs running the
// single-pair body on its arguments
__global__ void k_icp_begin_batch(const IcpJob* __restrict__ jobs, int n) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) icp_begin_body(jobs[v].st, jobs[v].guess);
}

__global__ void __launch_bounds__(kAssocThreads, 2) k_icp_step_batch(const IcpJob* __restrict__ jobs, BlockMap m) {
    const int v = block_owner(m, blockIdx.x);
    const unsigned int b0 = m.first[v];
    icp_step_body(jobs[v].a, jobs[v].st, blockIdx.x - b0, m.first[v + 1] - b0);
}

__global__ void k_backproject_batch(const BackprojectJob* __restrict__ jobs, BlockMap m) {
    const int v = block_owner(m, blockIdx.x);
    const BackprojectJob& j = jobs[v];
    const unsigned int b0 = m.first[v];
    backproject_body(j.depth, 1, j.width, j.height, j.fl_inv_x, j.fl_inv_y, j.pp_x, j.pp_y, j.e2w, j.out,
                     blockIdx.x - b0, m.first[v + 1] - b0);
}

// the same resolve into the association's float4 target layout
__global__ void k_bin_resolve_target(const float* __restrict__ pts, const unsigned long long* __restrict__ zbuf,
                                     int n_pix, float4* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pix; i += gridDim.x * blockDim.x) {
        const unsigned long long z = zbuf[i];
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        if (z != ~0ull) {
            const unsigned int j = (unsigned int)(z & 0xffffffffu);
            o = make_float4(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2], 0.f);
        }
        out[i] = o;
    }
}

}  // namespace

cudaError_t icp_align_enqueue(const IcpArgs& a, IcpState* st, const Mat4& guess, int iterations,
                              int /*ctas*/, cudaStream_t stream, IcpPoseMail* mail, unsigned long long seq) {
    k_icp_begin<<<1, 32, 0, stream>>>(st, guess);
    const int n_cols = (a.width + 3) / 4;
    const int tiles = ((n_cols + kTileCols - 1) / kTileCols) * ((a.height + kTileRows - 1) / kTileRows);
    const int ctas = tiles < kIcpMaxCtas ? tiles : kIcpMaxCtas;
    const size_t smem = 3 * kStagePixels * sizeof(float);
    // programmatic dependent launch: each step's grid is scheduled as soon as
    // every CTA of the one before has finished its association, overlapping
    // its launch with the previous finisher (k_icp_step waits for it)
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kAssocThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    IcpArgs last = a;  // the last step publishes the pose
    last.mail = mail;
    last.mail_seq = seq;
    IcpArgs other = a;
    other.mail = nullptr;
    for (int it = 0; it < iterations; ++it) {
        const cudaError_t e = cudaLaunchKernelEx(&cfg, k_icp_step, it + 1 == iterations ? last : other, st);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// The association's dynamic shared memory above the default 48 KB limit; set
// once per device, outside any stream capture.
cudaError_t icp_init_device() {
    cudaError_t e = cudaFuncSetAttribute(k_icp_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(3 * kStagePixels * sizeof(float)));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_icp_step_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(3 * kStagePixels * sizeof(float)));
    return e;
}

cudaError_t icp_align_batch_enqueue(const IcpJob* jobs, int n, const BlockMap& map, int iterations,
                                    cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_icp_begin_batch<<<(n + 63) / 64, 64, 0, stream>>>(jobs, n);
    const size_t smem = 3 * kStagePixels * sizeof(float);
    // programmatic dependent launch, as for a single pair: each step's grid
    // is scheduled once every CTA of the step before has finished its association
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(map.grid);
    cfg.blockDim = dim3(kAssocThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    for (int it = 0; it < iterations; ++it) {
        const cudaError_t e = cudaLaunchKernelEx(&cfg, k_icp_step_batch, jobs, map);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

cudaError_t backproject_batch_enqueue(const BackprojectJob* jobs, int n, const BlockMap& map, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_backproject_batch<<<map.grid, kThreads, 0, st>>>(jobs, map);
    return cudaGetLastError();
}

// CTAs of one pair's association (its tiles, at most kIcpMaxCtas)
int icp_tiles(int width, int height) {
    const int n_cols = (width + 3) / 4;
    const int tiles = ((n_cols + kTileCols - 1) / kTileCols) * ((height + kTileRows - 1) / kTileRows);
    return tiles < kIcpMaxCtas ? tiles : kIcpMaxCtas;
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

cudaError_t bin_target_enqueue(const float* pts, unsigned int n, const Mat4& w2c, int width, int height,
                               unsigned long long* zbuf, float4* out, int ctas, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(zbuf, 0xff, (size_t)width * height * 8, st);
    if (e) return e;
    if (n) k_bin_splat<<<ctas, kThreads, 0, st>>>(pts, n, w2c, width, height, zbuf);
    k_bin_resolve_target<<<ctas, kThreads, 0, st>>>(pts, zbuf, width * height, out);
    return cudaGetLastError();
}

}  // namespace kifi
