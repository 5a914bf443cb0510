// kifi_internal.h -- declarations shared between the library's translation
// units (not part of the public ABI).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "kifi_common.cuh"

namespace kifi {

// ------------------------------------------------------------ radix sort
// up to 8 digit passes: keys of up to 64 bits
constexpr int kSortMaxPasses = 8;
// A frame's 30-bit new keys sort in three 10-bit digit passes.  The frame's
// set-up kernel zeroes their histograms and tile counters, and the splat
// counts the digits of every key it stores, so the sort itself is the three
// passes (its result lands in SortScratch::alt_keys).
constexpr int kFrameDigitBits = 10;
constexpr int kFrameRadix = 1 << kFrameDigitBits;
constexpr int kFrameSortPasses = 3;
// counters of the largest digit set: 3 x 1024 (frame keys) or 8 x 256
constexpr int kSortHistWords = kFrameSortPasses * kFrameRadix;
static_assert(kSortHistWords >= kSortMaxPasses * 256, "histogram sized for both digit sets");
struct SortScratch {
    unsigned int* hist = nullptr;           // [passes][radix] digit counts
    unsigned int* tile_counter = nullptr;   // [passes] dynamic tile ids per pass
    unsigned long long* epoch = nullptr;    // look-back generation tag
    unsigned long long* lookback = nullptr; // [passes][max_tiles][radix]
    void* alt_keys = nullptr;               // ping-pong buffers, max_n (+pad), 8 bytes per key
    uint32_t* alt_vals = nullptr;
    unsigned int* status = nullptr;         // where timeouts are reported
    size_t max_tiles = 0, max_n = 0;
    // polls of a predecessor's look-back word before a pass gives up, and the
    // first tile id the passes hand out (0; a test sets both through
    // kifi_sort_set_fault_injection to make a look-back wait run out)
    unsigned long long spin_limit = 0;
    unsigned int first_tile = 0;
};

size_t sort_max_tiles(size_t max_n);
// zeroes its look-back words on `st`: the sorts that use it must run on st
// (or after it)
cudaError_t sort_scratch_alloc(SortScratch* s, size_t max_n, cudaStream_t st);
void sort_scratch_free(SortScratch* s);
cudaError_t sort_u32(uint32_t* keys, uint32_t* vals, const unsigned int* n_dev, SortScratch& s,
                     unsigned int* status, int grid_ctas, cudaStream_t st);
// keys of key_bytes (4 or 8) bytes holding key_bits significant bits: one
// stable 8-bit digit pass per byte of significant bits, rounded up to an
// even count so the result lands back in `keys`
cudaError_t sort_keys(void* keys, int key_bytes, int key_bits, uint32_t* vals, const unsigned int* n_dev,
                      SortScratch& s, unsigned int* status, int grid_ctas, cudaStream_t st);
// the frame path's three 10-bit passes over 30-bit keys whose histograms and
// pass counters are already set (see kFrameDigitBits); *sorted receives the
// buffer holding the result
cudaError_t sort_frame_keys(uint32_t* keys, const unsigned int* n_dev, SortScratch& s, unsigned int* status,
                            int grid_ctas, cudaStream_t st, const uint32_t** sorted);

// ------------------------------------------------------------- integrate
struct VolumeBuffers {
    int key_bytes = 4;              // 4: 30-bit keys (uint32_t), 8: 64-bit keys (uint64_t)
    void* keys[2] = {nullptr, nullptr};
    float2* vals[2] = {nullptr, nullptr};
    size_t cap = 0;                 // voxels per buffer (arrays hold cap + pad)
    uint32_t* bitmap = nullptr;     // res^3 occupancy bits
    size_t bitmap_words = 0;
    void* new_keys = nullptr;       // keys new to the volume in this frame
    uint32_t* new_idx = nullptr;    // insert path: source position of each new key
    size_t new_cap = 0;
    unsigned long long* splits = nullptr;  // merge-path split of every output tile
};

struct LaunchShape {
    int sms = 0;          // multiprocessors of the device
    int sort_ctas = 0;    // persistent CTAs of the sort passes
    int merge_ctas = 0;   // persistent CTAs of the merge/update kernel
    int splat_ctas = 0;
    // beside tracking (a pipeline's volume): short-lived CTAs and the merge
    // variant that leaves room on the SMs (3 CTAs of 256 threads per SM);
    // alone: persistent CTAs and the merge variant capped at 64 registers
    // (4 CTAs per SM)
    bool beside_tracking = false;
};

// Enqueues one Integrator::Integrate on `st`.  depth_dev holds the frame
// (float metres, or uint16 millimetres when depth_u16).
// `events` (optional, 4 entries) are recorded before the frame set-up, after
// splat+emit, after the sort and after merge+update.
cudaError_t integrate_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb, SortScratch& ss,
                              const void* depth_dev, bool depth_u16, const kifi_camera& cam,
                              const Mat4& world_to_eye, const LaunchShape& ls, cudaStream_t st,
                              cudaEvent_t* events);

// resident CTAs per SM of the merge/update kernel (occupancy API)
int merge_blocks_per_sm();

// flat_map::insert of n sorted unique device keys: filter out resident keys
// (their values win) and collect (key, index) of the rest in new_keys /
// new_idx; the caller sorts those pairs and then merges.
// merge-path split slots a volume of `cap` voxels needs
size_t merge_max_tiles(const VolumeBuffers& vb, size_t cap);
cudaError_t insert_filter_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                  const void* keys_dev, const unsigned int* n_dev,
                                  const LaunchShape& ls, cudaStream_t st);
cudaError_t insert_merge_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                 const float2* vals_dev, const LaunchShape& ls, cudaStream_t st);
// clears the occupancy bitmap and sets the bits of the resident keys
cudaError_t bitmap_rebuild_enqueue(const DeviceCtl* ctl, const Geom& g, const VolumeBuffers& vb,
                                   const LaunchShape& ls, cudaStream_t st);

// ------------------------------------------------------------- batches
// A batched launch runs one stage for several volumes (or ICP frame pairs)
// at once: volume v owns the CTAs [first[v], first[v+1]) of the grid and
// reads its arguments from a device table.
struct BlockMap {
    const unsigned int* first;  // device, n + 1 entries; first[n] = grid
    int n;
    unsigned int grid;          // the launch's CTAs (known on the host)
};

// One volume's frame in a batched fusion launch: the arguments of the
// single-volume kernels.  Depth frames are uint16 millimetres.
struct FuseJob {
    DeviceCtl* ctl;
    Geom g;
    VolumeBuffers vb;
    SortScratch ss;
    const void* depth;
    FrameConst fc;
    unsigned int max_tiles;  // merge-path split slots of the volume
};

#ifdef __CUDACC__
// the volume that owns CTA b of a batched launch
__device__ __forceinline__ int block_owner(const BlockMap& m, unsigned int b) {
    int lo = 0, hi = m.n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (m.first[mid] <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}
#endif

// The CTA shares of one batched fusion step, one map per stage; every
// volume of the batch has the same key width.
struct FuseMaps {
    BlockMap splat, hist, pass, partition, merge;
};

// The batched fusion of a step as one persistent launch over a device work
// queue (integrate_queue_enqueue): stages 0 set-up, 1 splat, 2 histogram,
// 3 .. 2 + passes the digit passes, then the partition and the merge; first[k]
// is the number of stage k's first item, first[stages] the item count.
constexpr int kQueueMaxStages = 5 + kSortMaxPasses;
struct FuseQueuePlan {
    int n = 0;       // scenes
    int passes = 0;  // digit passes
    int stages = 0;  // 5 + passes
    unsigned int first[kQueueMaxStages + 1] = {};
    BlockMap maps[5] = {};  // splat, histogram, pass, partition, merge
};
// the block map of stage k (k >= 1)
KIFI_HD int fuse_stage_map(int k, int passes) {
    return k == 1 ? 0 : k == 2 ? 1 : k < 3 + passes ? 2 : k == 3 + passes ? 3 : 4;
}

// Enqueues Integrator::Integrate of one frame for each of the n volumes of
// `jobs` (a device table) on `st`: one launch per stage for all of them.
// key_bytes: the volumes' key width; passes: digit passes of the sort.
// the sort of every volume's new keys (FuseJob::vb.new_keys, count in ctl->n_new)
cudaError_t sort_batch_enqueue(const FuseJob* jobs, int n, int key_bytes, int passes, const BlockMap& hist,
                               const BlockMap& pass, cudaStream_t st);
// the look-back limits every sort applies (kifi_sort_set_fault_injection)
void sort_limits(SortScratch* s);
cudaError_t integrate_batch_enqueue(const FuseJob* jobs, int n, int key_bytes, int passes, const FuseMaps& maps,
                                    cudaStream_t st);
// the same as one persistent launch of `ctas` CTAs; next (1 word) and done
// (plan.n x plan.stages words) must be zero
cudaError_t integrate_queue_enqueue(const FuseJob* jobs, int key_bytes, const FuseQueuePlan& plan,
                                    unsigned int* next, unsigned int* done, int ctas, cudaStream_t st);

// ---------------------------------------------------------------- mesher
struct MeshCounts {
    unsigned long long n_verts;
    unsigned long long n_idx;
    unsigned long long missing_min;  // smallest triangle edge id without a vertex (or ~0)
    unsigned long long overflow;     // emission skipped: the output buffers were too small
    unsigned long long n_flagged;    // voxels with output (vertices or triangles)
    unsigned long long error;        // non-zero: a bounded wait of the classification gave up
};

// per classification tile: the voxels staged for its lookups -- region A,
// from the tile's first voxel on (the tile itself and its +y lookups), and
// region B (the +z and +yz lookups) in up to two ranges (lo, len), the second
// for the tile's voxels from `split` on (split = the tile's end when there is
// one range)
struct MeshTileRange {
    unsigned int a_len, b_lo[2], b_len[2], split;
};

struct MeshScratch {
    // per voxel: vertex axes | triangle count << 3 | marching-cubes case << 6 |
    // the voxel's first vertex within its classification tile << 14
    unsigned int* vflags = nullptr;
    unsigned char* vstatus = nullptr;      // per voxel: the status byte classification reads
    // per voxel with output: indices of its +y, +z, +yz lookups and its first
    // index within its classification tile
    uint4* corners = nullptr;
    // per classification tile: packed (index count << 32 | vertex count),
    // then (after the scan) their exclusive prefix
    unsigned long long* tile_sums = nullptr;
    // per tile: its voxels with output, then (after the scan) their exclusive
    // prefix, with the total at [tiles]
    unsigned int* tile_nflag = nullptr;
    unsigned int* flagged = nullptr;       // per tile, a slot per voxel: those voxels, ascending
    unsigned int* rows = nullptr;          // start index of each (z, y) key row
    MeshTileRange* tile_ranges = nullptr;  // per classification tile: the staged regions
    MeshCounts* counts = nullptr;
    unsigned int* n_dev = nullptr;         // the voxel count the passes read
    size_t cap = 0, rows_cap = 0;
};

cudaError_t mesh_scratch_reserve(MeshScratch* m, size_t n, int kb);
void mesh_scratch_free(MeshScratch* m);
// stage_events (optional, 2 entries): recorded after the row directory and
// after the classification
cudaError_t mesh_count_enqueue(const void* keys, int key_bytes, const float2* vals, size_t n_cap, int kb,
                               int with_indices, MeshScratch& ms, int sms, cudaStream_t st,
                               cudaEvent_t* stage_events = nullptr);
// Emission reads the counts on the device (ms.counts, written by the
// counting passes), so it can be enqueued right behind them.  The buffers
// hold vert_cap vertices and idx_cap indices; when the mesh needs more, the
// emission writes nothing and sets ms.counts->overflow instead.
cudaError_t mesh_emit_enqueue(const Geom& g, const void* keys, int key_bytes, const float2* vals, size_t n_cap,
                              int with_indices, MeshScratch& ms, size_t vert_cap, size_t idx_cap,
                              float* verts_dev, uint32_t* idx_dev, int sms, cudaStream_t st);
cudaError_t mesh_snapshot_enqueue(const DeviceCtl* ctl, const VolumeBuffers& vb, void* keys, float2* vals,
                                  size_t cap, unsigned int* n_dev, int sms, cudaStream_t st);

// ------------------------------------------------------------------ ICP
constexpr int kIcpMaxStats = 64;
constexpr int kIcpMaxCtas = 2048;

// Where the last step of an alignment publishes its pose for a host that
// polls instead of synchronising (page-locked, mapped host memory): the pose
// (kifi order), then the alignment's sequence number, written after it.
struct IcpPoseMail {
    float pose[16];
    unsigned long long seq;
};

struct IcpArgs {
    const void* depth;      // source frame (float metres or uint16 mm)
    int depth_u16;
    int width, height;
    float fl_inv_x, fl_inv_y, pp_x, pp_y;
    float proj[16];         // EyeToClipRH * inverse(synth eye-to-world), kifi order
    const float4* synth;    // target world points (w unused), synth_w * synth_h
    int synth_w, synth_h;
    long long* pairs;       // optional: per source the winner's target index (-1: none) ...
    float* pairs_len2;      // ... and its len^2, overwritten by every iteration
    float neg_zero;         // -0.0f, a value the device code cannot see at compile time
    IcpPoseMail* mail;      // the step that publishes the final pose (the last): its
    unsigned long long mail_seq;  // mailbox and the alignment's number; null otherwise
};

struct IcpIterStats {
    int n_assoc;
    int solver;       // Horn's eigenvector: 0 closed form, 1 Jacobi fallback
    float sum_l2;     // the associated squared distances' sum (the host forms the RMS)
    float body_us;    // first CTA start to last CTA end of the association
    float tail_us;    // last CTA end to the updated pose
};

struct IcpState {
    float pose_f[16];   // eye-to-world estimate, kifi order (float-float high part)
    float pose_lo[16];  // and its low part
    unsigned long long done;  // CTAs finished (high 32 bits) and their associations (low 32 bits)
    float mu_s[4], mu_d[4];
    int n_assoc;
    int iter;
    unsigned long long t_start, t_body;  // globaltimer stamps of the running step
    IcpIterStats stats[kIcpMaxStats];
    float part[34 * kIcpMaxCtas];   // per-CTA float-float partials: hi, lo rows of 17 components
    int tile_box[4 * kIcpMaxCtas];  // each tile's window box in the last step: x0, y0, x1, y1
};

cudaError_t icp_init_device();
// One ICP frame pair of a batched alignment: the arguments of the
// single-pair kernels.
struct IcpJob {
    IcpArgs a;
    IcpState* st;
    Mat4 guess;
};
// `iterations` AlignSteps of the n pairs of `jobs` (a device table), one
// launch per step for all of them; pair v's CTAs are map.first[v] ..
// map.first[v+1] - 1, one per association tile.
cudaError_t icp_align_batch_enqueue(const IcpJob* jobs, int n, const BlockMap& map, int iterations,
                                    cudaStream_t stream);
// Back-projection of one frame per pair into its target (the next frame's
// ICP target), for the n entries of `jobs` (device table).
struct BackprojectJob {
    const void* depth;  // uint16 millimetres
    int width, height;
    float fl_inv_x, fl_inv_y, pp_x, pp_y;
    Mat4 e2w;
    float4* out;
};
cudaError_t backproject_batch_enqueue(const BackprojectJob* jobs, int n, const BlockMap& map, cudaStream_t st);
// CTAs of one frame pair's association (one per tile)
int icp_tiles(int width, int height);
// mail (device address of mapped host memory, or null): the last step
// publishes the final pose there with sequence number `seq`
cudaError_t icp_align_enqueue(const IcpArgs& a, IcpState* st, const Mat4& guess, int iterations,
                              int ctas, cudaStream_t stream, IcpPoseMail* mail = nullptr,
                              unsigned long long seq = 0);
cudaError_t backproject_enqueue(const void* depth, bool u16, const kifi_camera& cam,
                                const Mat4& eye_to_world, float4* out, int ctas, cudaStream_t st);
cudaError_t expand_target_enqueue(const float* in, int n, float4* out, int ctas, cudaStream_t st);

cudaError_t bin_enqueue(const float* pts, unsigned int n, const Mat4& w2c, int width, int height,
                        unsigned long long* zbuf, float* out, int ctas, cudaStream_t st);
// Bin straight into an ICP target (float4 per pixel, w unused)
cudaError_t bin_target_enqueue(const float* pts, unsigned int n, const Mat4& w2c, int width, int height,
                               unsigned long long* zbuf, float4* out, int ctas, cudaStream_t st);

// Optional epilogue of gemm_bf16_enqueue: C = acc + bias[n] (FP32), or with
// out_bf16 set, out_bf16 = bf16(relu?(acc + bias[n])) (row stride ldc) in
// place of C.
struct GemmEpilogue {
    const float* bias = nullptr;
    bool relu = false;
    void* out_bf16 = nullptr;
};

// C[M x N] (+)= A[M x K] * B[N x K]^T, BF16 in, FP32 out, on tcgen05 tensor
// cores with TMA-fed operands (kifi_tc_gemm.cu).  k_split > 0 splits K
// across tiles that add into C atomically (atomic must then be true and C
// pre-initialised; the split is rounded up to a multiple of 64).
cudaError_t gemm_bf16_enqueue(const void* A, const void* B, float* C, int M, int N, int K, int lda, int ldb,
                              int ldc, int k_split, bool atomic, unsigned int* status, cudaStream_t st,
                              const GemmEpilogue* epi = nullptr);

// 3x3 / stride 2 / pad 1 convolution of an NHWC BF16 input [batch][H][W][Cin]
// (Cin 32 or 64) with weights [Co][Kp] (k = (ky * 3 + kx) * Cin + c, Co 64 or
// 128) as an implicit GEMM on the tensor cores: out_bf16 [batch][Ho][Wo][Co]
// = bf16(relu?(conv + bias)), Ho = (H + 1) / 2, Wo = (W + 1) / 2.
cudaError_t conv3x3s2_bf16_enqueue(const void* x, int batch, int H, int W, int Cin, const void* Wt, int Co, int Kp,
                                   const float* bias, bool relu, void* out_bf16, unsigned int* status,
                                   cudaStream_t st);

}  // namespace kifi
