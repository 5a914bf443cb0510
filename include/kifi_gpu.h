/*
 * kifi_gpu.h -- C ABI of the GB300 (sm_103a) depth-fusion library
 * (libkifi_gpu.so), a drop-in for the per-frame fusion path of
 * denniskb/merge_fusion's kifi library (KinectFission/kifi).
 *
 * Every entry point below names the reference interface it replaces.  The
 * reference has no FFI of its own; its boundary is the C++ class API that
 * kifi::Pipeline and the unit tests call.  include/kifi_gpu.hpp wraps these
 * functions in classes with the reference's names and signatures.
 *
 * Conventions
 *  - Plain pointers and sizes; no CUDA or C++ types in signatures.  A
 *    `stream` argument or field is a cudaStream_t passed as void*.
 *  - Matrices are 16 floats in kifi's util::float4x4 memory order: four
 *    columns of four floats (KinectFission/kifi/util/math.h:59-61), so a
 *    kifi float4x4 can be passed by address.
 *  - Volumes hold sorted 30-bit linear voxel keys, key = z<<20 | y<<10 | x
 *    (util::pack, math.h:442-445), and per voxel a (distance-sum, weight)
 *    pair of floats (kifi::Voxel, Voxel.h:9-21).
 *  - Every call returns a kifi_status; nothing throws across the ABI.  The
 *    reference signals misuse only through assert(); here misuse returns
 *    KIFI_ERR_INVALID_ARGUMENT.
 *  - Threading: a volume (or ICP context) is not safe for concurrent calls;
 *    different handles are independent.  All device work of a handle runs on
 *    its own CUDA stream.
 */
#ifndef KIFI_GPU_H
#define KIFI_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define KIFI_API __attribute__((visibility("default")))
#else
#define KIFI_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum kifi_status {
    KIFI_OK = 0,
    KIFI_ERR_INVALID_ARGUMENT = 1,
    KIFI_ERR_OUT_OF_MEMORY = 2,
    KIFI_ERR_CUDA = 3,
    KIFI_ERR_CAPACITY = 4,     /* an output buffer or volume capacity is too small */
    KIFI_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    KIFI_ERR_UNSUPPORTED = 6,
    KIFI_ERR_NO_DEVICE = 7,
    KIFI_ERR_IO = 8,
    KIFI_ERR_FORMAT = 9,
    KIFI_ERR_END_OF_STREAM = 10
} kifi_status;

/* Replaces kifi::DepthSensorParams (KinectFission/kifi/DepthSensorParams.h:23-52):
 * resolution, focal length and principal point in pixels, and the sensible
 * depth range in metres (used only by EyeToClipRH, DepthSensorParams.cpp:47-63). */
typedef struct kifi_camera {
    int width, height;
    float fx, fy;
    float cx, cy;
    float znear_m, zfar_m;
} kifi_camera;

/* Replaces the arguments of kifi::Volume::Volume(int resolution,
 * float sideLength, float truncationMargin) (KinectFission/kifi/Volume.h:15,
 * Volume.cpp:12-37).  resolution: power of two in [2, 1024].  The volume is a
 * cube of side_length_m centred at the world origin (Volume.cpp:63-71). */
typedef struct kifi_volume_desc {
    int resolution;
    float side_length_m;
    float truncation_m;
    size_t initial_capacity; /* voxels to reserve up front; 0 = library default */
    int device;              /* CUDA device ordinal */
    void* stream;            /* cudaStream_t to run on, or NULL for a library-owned stream */
    int key_bits;            /* 0: 32 up to 1024 voxels per axis, else 64; 32 or 64 to choose.
                              * 32-bit keys are util::pack (math.h:442-457), z<<20|y<<10|x;
                              * 64-bit keys are z<<2b|y<<b|x with b = max(10, log2 resolution),
                              * so below 1024 voxels per axis both name a voxel alike. */
} kifi_volume_desc;

typedef struct kifi_volume kifi_volume;

/* Human-readable name of a status code. */
KIFI_API const char* kifi_status_string(kifi_status status);

/* Detail of the last failing call on this thread (empty when none). */
KIFI_API const char* kifi_last_error(void);

/* Number of CUDA devices visible to the library (0 when there is none). */
KIFI_API kifi_status kifi_device_count(int* count);

/* kifi::Volume::Volume (Volume.h:15).  Allocates the device-resident sorted
 * key/value arrays and the occupancy bitmap of the volume. */
KIFI_API kifi_status kifi_volume_create(const kifi_volume_desc* desc, kifi_volume** out);

/* kifi::Volume::~Volume */
KIFI_API kifi_status kifi_volume_destroy(kifi_volume* vol);

/* kifi::Volume::Data().size() (flat_map.h:199-203).  Waits for queued work. */
KIFI_API kifi_status kifi_volume_size(kifi_volume* vol, size_t* n);

/* Reads the volume back: the sorted keys (flat_map keys_cbegin..keys_cend,
 * flat_map.h:27-30) and the voxels as (distance-sum, weight) float pairs
 * (values_cbegin.., flat_map.h:32-37).  On KIFI_ERR_CAPACITY *n holds the
 * size needed.  Waits for queued work. */
KIFI_API kifi_status kifi_volume_export(kifi_volume* vol, uint32_t* keys, float* values, size_t capacity,
                               size_t* n);

/* kifi_volume_export with 64-bit keys (any volume). */
KIFI_API kifi_status kifi_volume_export64(kifi_volume* vol, uint64_t* keys, float* values, size_t capacity,
                                          size_t* n);

/* The volume's key width (32 or 64) and key bits per axis (b). */
KIFI_API kifi_status kifi_volume_key_bits(kifi_volume* vol, int* key_bits, int* bits_per_axis);

/* kifi::util::flat_map::insert (flat_map.h:164-197) on the volume's map:
 * the set union of the resident voxels with `keys` (sorted, unique), where
 * resident voxels keep their value.  values may be NULL for Voxel() = (0,0),
 * as Integrator::Integrate inserts (Integrator.cpp:60-63). */
KIFI_API kifi_status kifi_volume_insert(kifi_volume* vol, const uint32_t* keys, const float* values,
                               size_t n);

/* kifi_volume_insert with 64-bit keys (any volume). */
KIFI_API kifi_status kifi_volume_insert64(kifi_volume* vol, const uint64_t* keys, const float* values,
                                          size_t n);

/* kifi::util::flat_map::clear (flat_map.h:157-162) */
KIFI_API kifi_status kifi_volume_clear(kifi_volume* vol);

/* Grows the device capacity to at least `capacity` voxels (no reference
 * counterpart: flat_map grows its std::vectors implicitly). */
KIFI_API kifi_status kifi_volume_reserve(kifi_volume* vol, size_t capacity);

/* Waits for the volume's stream and reports any error raised on the device
 * by asynchronous calls since the last sync. */
KIFI_API kifi_status kifi_volume_sync(kifi_volume* vol);

/* The cudaStream_t (as void*) the volume's device work runs on. */
KIFI_API void* kifi_volume_stream(kifi_volume* vol);

/* kifi::Integrator::Integrate(Volume&, vector2d<float> const& frame,
 * DepthSensorParams const&, float4x4 const& worldToEye)
 * (KinectFission/kifi/Integrator.h:19-26, Integrator.cpp:26-71): splat the
 * frame's pixels to voxel keys, dilate them by {0,1}^3, merge them into the
 * resident volume and update the TSDF of every resident voxel.
 * depth_m: width*height floats, row-major, metres, 0 = no measurement.
 * Synchronous: returns when the volume is updated. */
KIFI_API kifi_status kifi_integrate_f32(kifi_volume* vol, const float* depth_m, const kifi_camera* cam,
                               const float world_to_eye[16]);

/* Same, from 16-bit millimetre texels converted exactly as
 * kifi::DepthStream::NextFrame does (value * 0.001f, DepthStream.cpp:81-92). */
KIFI_API kifi_status kifi_integrate_u16(kifi_volume* vol, const uint16_t* depth_mm, const kifi_camera* cam,
                               const float world_to_eye[16]);

/* Same, with the frame already in device memory (float metres, or uint16
 * millimetres when depth_is_u16 != 0).  Asynchronous: only enqueues work on
 * the volume's stream; errors surface at kifi_volume_sync. */
KIFI_API kifi_status kifi_integrate_device(kifi_volume* vol, const void* depth_dev, int depth_is_u16,
                                  const kifi_camera* cam, const float world_to_eye[16]);

/* kifi::Mesher::Mesh (KinectFission/kifi/Mesher.h:17-18, Mesher.cpp:14-45):
 * sparse marching cubes over the resident voxels.
 * with_indices = 0: Mesh(volume, verts) -- vertices only, in the reference's
 *   generation order; indices is not written.
 * with_indices = 1: Mesh(volume, verts, indices) -- vertices ordered by
 *   their edge id, triangle indices in generation order.
 * verts receives 3 floats per vertex.  When a capacity is too small the call
 * returns KIFI_ERR_CAPACITY with the required counts in *n_verts/*n_indices
 * and writes nothing. */
KIFI_API kifi_status kifi_mesh(kifi_volume* vol, int with_indices, float* verts, size_t vert_capacity,
                      uint32_t* indices, size_t index_capacity, size_t* n_verts,
                      size_t* n_indices);

/* Mesher::Mesh into device memory owned by the volume: the same output as
 * kifi_mesh, left on the GPU.  *verts_dev / *indices_dev stay valid until
 * the next mesh call on the volume or its destruction.  Either pointer
 * argument may be NULL. */
KIFI_API kifi_status kifi_mesh_device(kifi_volume* vol, int with_indices, size_t* n_verts,
                                      size_t* n_indices, const float** verts_dev,
                                      const uint32_t** indices_dev);

/* Stage timers, the GPU counterpart of the stop_watch the reference wires
 * into Integrator::Integrate (Integrator.cpp:45-70, "tmerge"/"tupd"): while
 * on, every integrated frame records CUDA events around splat+emit, the sort
 * of the new keys, the merge partition and the fused merge+update.
 * kifi_volume_stage_times waits for them, returns the summed milliseconds of
 * the four stages and the number of frames, and resets the accumulation. */
KIFI_API kifi_status kifi_volume_set_profiling(kifi_volume* vol, int on);
KIFI_API kifi_status kifi_volume_stage_times(kifi_volume* vol, double out_ms[4], int* frames);
/* No counterpart in the reference.  While profiling is on, kifi_mesh and
 * kifi_mesh_device time the device work of each mesh (counting passes and
 * emission); this returns their mean in milliseconds and their count, and
 * resets them. */
KIFI_API kifi_status kifi_volume_mesh_times(kifi_volume* v, double* out_ms, int* meshes);
/* The same per stage: out_ms = {row directory, classification, scan,
 * emission, total} means in milliseconds. */
KIFI_API kifi_status kifi_volume_mesh_stage_times(kifi_volume* v, double out_ms[5], int* meshes);

/* No counterpart in the reference.  The volume's launch shape: beside
 * tracking (beside_tracking != 0; what a pipeline gives its volume) the
 * fusion kernels run as short-lived CTAs and the merge/update as its build
 * that holds fewer SM resources, so that ICP steps find free SMs; alone
 * (0, the default) as persistent CTAs and the merge/update build with more
 * CTAs per SM.  Results are identical either way.  Resets any autotuned
 * CTA counts. */
KIFI_API kifi_status kifi_volume_set_launch_mode(kifi_volume* vol, int beside_tracking);

/* No counterpart in the reference.  Picks the persistent CTA counts of the
 * volume's splat+emit, sort and merge/update kernels by timing them on one
 * frame (device memory) integrated from a snapshot of the volume, which is
 * restored: the volume is unchanged and later results are identical for any
 * choice.  The choice is cached per (GPU, resolution, frame size) for the
 * process and, when the environment variable KIFI_AUTOTUNE_CACHE names a
 * file, there; force != 0 re-measures.  out_ctas (may be NULL) receives the
 * splat, sort and merge CTA counts. */
KIFI_API kifi_status kifi_volume_autotune(kifi_volume* vol, const void* depth_dev, int depth_is_u16,
                                          const kifi_camera* cam, const float world_to_eye[16], int force,
                                          int out_ctas[3]);

/* Sizes of the most recent merges (up to 64, oldest first): resident voxels
 * before, keys new to the volume, resident voxels after.  No reference
 * counterpart; it sizes the bytes each merge moves. */
KIFI_API kifi_status kifi_volume_frame_log(kifi_volume* vol, uint64_t* n_before, uint64_t* n_new,
                                           uint64_t* n_after, int capacity, int* count);

/* kifi::util::radix_sort(T* first, T* last, void* scratch)
 * (KinectFission/kifi/util/algorithm.h:63-91) on the GPU: stable LSD sort of
 * n 32-bit keys held in host memory, in place. */
KIFI_API kifi_status kifi_radix_sort_u32(uint32_t* keys, size_t n);

/* kifi::util::radix_sort(keys, keys_last, values, scratch)
 * (algorithm.h:93-134): stable sort of 32-bit keys carrying 32-bit values. */
KIFI_API kifi_status kifi_radix_sort_pairs_u32(uint32_t* keys, uint32_t* values, size_t n);

/* The same radix sort widened to 64-bit keys (eight 8-bit digit passes),
 * the sort behind volumes with 64-bit keys. */
KIFI_API kifi_status kifi_radix_sort_u64(uint64_t* keys, size_t n);
KIFI_API kifi_status kifi_radix_sort_pairs_u64(uint64_t* keys, uint32_t* values, size_t n);

/* No counterpart in the reference: fault injection for the failure-detection
 * tests.  Every sort's digit passes resolve their offsets by a bounded wait
 * on the look-back words of the tiles before them.  After this call, the
 * sorts enqueued in this process hand out tile ids from skip_tiles on (so
 * tiles below it are never processed and the waits on them cannot end) and
 * give up a wait after spin_limit polls, raising KIFI_ERR_TIMEOUT; every
 * store stays inside the output buffers.  (0, 0) restores the defaults (no
 * skipped tile, 2^22 polls).  Not for production use. */
KIFI_API kifi_status kifi_sort_set_fault_injection(unsigned int skip_tiles, unsigned long long spin_limit);

/* No counterpart in the reference.  The radix sort of
 * kifi_radix_sort_pairs_u32 for callers that must not allocate device
 * memory: it sorts keys_dev[0..n) -- and values_dev[0..n) with them when
 * values_dev is not NULL -- in place, in device memory, on `stream` (a
 * cudaStream_t; NULL for the default stream), with results identical to
 * kifi_radix_sort_pairs_u32.  Its scratch is a fixed area of static device
 * memory built into the library (12.0 MiB, present once the library's
 * module is loaded); it calls no cudaMalloc, cudaFree or other allocating
 * routine.  It is meant for processes whose device memory is handed out by
 * their own pool, and for frame loops that cannot pay for cudaMalloc /
 * cudaFree, which synchronise the device and stall its other streams.
 *  - n <= KIFI_RADIX_SORT_STATIC_MAX; a larger n returns
 *    KIFI_ERR_INVALID_ARGUMENT and does nothing.
 *  - The first call on a device (the device current at the call) looks up
 *    the scratch area's address; make that first call before any stream
 *    capture.  The address is kept for the life of the process:
 *    cudaDeviceReset (or another context on that device) invalidates it.
 *  - Every call waits on the host for its sort to finish and reads the
 *    device status word back before it returns.
 *  - There is one scratch area per device: calls that overlap in time (from
 *    several host threads, or on several streams) race on it and corrupt
 *    each other's results.  Serialise them.  The call returns only when the
 *    sort has finished on `stream`, so calls made one after another from
 *    one thread never overlap.
 *  - The caller zeroes nothing: the scratch state that must start at zero
 *    is zero when the library is loaded, and the rest is reset by each call.
 *  - KIFI_ERR_TIMEOUT when a bounded device wait gave up. */
#define KIFI_RADIX_SORT_STATIC_MAX (1u << 20)
KIFI_API kifi_status kifi_radix_sort_pairs_u32_static(uint32_t* keys_dev, uint32_t* values_dev, size_t n,
                                                      void* stream);

/* ------------------------------------------------------------------ ICP */

/* Context of kifi::ICP (KinectFission/kifi/ICP.h:15-42): device buffers for
 * the source frame, the target point buffer and the association pairs, and
 * the pose estimate (kept in double on the device). */
typedef struct kifi_icp kifi_icp;

KIFI_API kifi_status kifi_icp_create(int device, void* stream, kifi_icp** out);
KIFI_API kifi_status kifi_icp_destroy(kifi_icp* icp);
KIFI_API void* kifi_icp_stream(kifi_icp* icp);

/* Diagnostics of ICP::AlignStep's association (ICP.cpp:66-131; no reference
 * accessor).  While recording is on, every iteration stores per source
 * pixel (rows, then every 4th column) the linear index y1 * width + x1 of
 * its nearest target point, or -1 when it has none (also for pixels without
 * depth), and that point's squared distance (0.01 when none).
 * kifi_icp_associations reads back the last iteration's; *n = sources. */
KIFI_API kifi_status kifi_icp_record_associations(kifi_icp* icp, int on);
KIFI_API kifi_status kifi_icp_associations(kifi_icp* icp, int64_t* target_index, float* len2, size_t capacity,
                                           size_t* n);

/* The synthetic target of ICP::Align (ICP.h:23-24): a width x height
 * row-major buffer of world points (3 floats each, (0,0,0) = no point) and
 * the eye-to-world pose of the camera that produced it. */
KIFI_API kifi_status kifi_icp_set_target(kifi_icp* icp, const float* points, int width, int height,
                                         const float synth_eye_to_world[16]);

/* Renderer::Bin of device-resident world points (3 floats each) straight
 * into the ICP target: the z-buffered splat through world_to_clip into a
 * width x height target, as the reference's tracking pipeline renders its
 * mesh for the next ICP::Align (Pipeline.cpp:48-52 then :38).  Asynchronous
 * on the ICP stream: the points must stay valid until that stream has run
 * it. */
KIFI_API kifi_status kifi_icp_set_target_bin_device(kifi_icp* icp, const float* points_dev, size_t n,
                                                    const float world_to_clip[16], int width, int height,
                                                    const float synth_eye_to_world[16]);

/* Target from a depth frame (host or device memory): every pixel
 * back-projected to world space with the frame's eye-to-world pose, using
 * the back-projection of Integrator::DepthMap2PointCloud
 * (Integrator.cpp:121-144) -- "ICP between consecutive frames". */
KIFI_API kifi_status kifi_icp_set_target_from_depth(kifi_icp* icp, const void* depth, int on_device,
                                                    int depth_is_u16, const kifi_camera* cam,
                                                    const float eye_to_world[16]);

/* kifi::ICP::Align (ICP.h:18-27, ICP.cpp:9-31) against the current target,
 * with a caller-chosen iteration count (the reference fixes 4): each
 * iteration is one AlignStep (ICP.cpp:35-265) -- projective association in a
 * 21x21 window, Horn's closed form -- and the step is left-multiplied onto
 * the pose.  depth_m: host float metres.  Synchronous. */
KIFI_API kifi_status kifi_icp_align(kifi_icp* icp, const float* depth_m, const kifi_camera* cam,
                                    const float eye_to_world_guess[16], int iterations,
                                    float out_eye_to_world[16]);

/* Same on a device-resident frame; asynchronous (read with kifi_icp_result). */
KIFI_API kifi_status kifi_icp_align_device(kifi_icp* icp, const void* depth_dev, int depth_is_u16,
                                           const kifi_camera* cam,
                                           const float eye_to_world_guess[16], int iterations);

/* Waits and reads the last alignment: the pose (float, and optionally the
 * float-float value it was rounded from, as a double), per-iteration
 * association counts and RMS
 * residuals (up to `capacity` entries; the reference prints the count,
 * ICP.cpp:133) and the iteration count.  Pointers may be NULL. */
KIFI_API kifi_status kifi_icp_result(kifi_icp* icp, float out_eye_to_world[16],
                                     double out_eye_to_world_d[16], int* n_assoc, double* rms,
                                     int capacity, int* iterations);

/* Per-iteration device timings of the last alignment (the GPU counterpart
 * of the reference's stop_watch telemetry): microseconds from the first CTA's
 * start to the last CTA's end of the association, and from there to the
 * updated pose (the reduction and Horn solve).  Pointers may be NULL. */
KIFI_API kifi_status kifi_icp_iteration_times(kifi_icp* icp, float* body_us, float* tail_us,
                                              int capacity, int* iterations);

/* kifi::Renderer::Bin (KinectFission/kifi/Renderer.h:23-29,
 * Renderer.cpp:39-80): z-buffered splat of n world points (3 floats each,
 * host memory) through world_to_clip into a width x height float3 buffer;
 * per pixel the first point with the smallest clip z wins, empty pixels are
 * (0,0,0). */
KIFI_API kifi_status kifi_bin(const float* points, size_t n, const float world_to_clip[16],
                              float* out, int width, int height);

/* ----------------------------------------------------------------- I/O */

/* kifi::DepthStream (KinectFission/kifi/DepthStream.h:13-45,
 * DepthStream.cpp:15-102): a .depth v1 (640x480, 16-bit mm) or v2 (width,
 * height, 16-bit mm or float m) recording.  Header errors return
 * KIFI_ERR_FORMAT (the reference asserts). */
typedef struct kifi_depthstream kifi_depthstream;
KIFI_API kifi_status kifi_depthstream_open(const char* path, kifi_depthstream** out);
KIFI_API kifi_status kifi_depthstream_close(kifi_depthstream* stream);
/* DepthStream::FrameCount (DepthStream.h:24) plus the frame geometry */
KIFI_API kifi_status kifi_depthstream_info(kifi_depthstream* stream, int* width, int* height,
                                           int* texel_is_u16, int* frame_count);
/* DepthStream::NextFrame (DepthStream.cpp:55-98): the next frame as float
 * metres (width*height, row-major; 16-bit texels * 0.001f) and its view
 * matrix (world to eye, kifi column order).  KIFI_ERR_END_OF_STREAM after
 * the last frame (the reference returns false); KIFI_ERR_FORMAT on a
 * truncated frame. */
KIFI_API kifi_status kifi_depthstream_next_frame(kifi_depthstream* stream, float* out_depth_m,
                                                 float out_view[16]);
/* The same frame copied raw -- 16-bit millimetres or float metres, as
 * kifi_depthstream_info reports -- into device memory, asynchronously on
 * `stream` (a cudaStream_t) through pinned double-buffered staging; pass the
 * buffer to the *_device integrate calls with the matching depth_is_u16.
 * The view is returned at once. */
KIFI_API kifi_status kifi_depthstream_next_frame_device(kifi_depthstream* stream, void* depth_dev,
                                                        float out_view[16], void* cuda_stream);

/* kifi::Mesher::Mesh2Obj (Mesher.h:20-25, Mesher.cpp:50-78): "v x y z" lines
 * (printf %f) then "f a b c" lines with 1-based indices. */
KIFI_API kifi_status kifi_mesh_to_obj(const float* verts, size_t n_verts, const uint32_t* indices,
                                      size_t n_indices, const char* path);

/* Volume checkpoints; no counterpart in the reference.  kifi_volume_save
 * writes the geometry, the sorted keys and the (distance-sum, weight) voxels;
 * kifi_volume_load creates a volume on `device` holding exactly those
 * voxels, so integration resumes where it stopped. */
KIFI_API kifi_status kifi_volume_save(kifi_volume* vol, const char* path);
KIFI_API kifi_status kifi_volume_load(const char* path, int device, kifi_volume** out);

/* ------------------------------------------------------- learned proposer */

/* No counterpart in the reference.  The pose proposer's tensor-core GEMM:
 * C[m x n] = A[m x k] * B[n x k]^T (or C += with accumulate != 0), A and B
 * BF16 in device memory with K contiguous (row strides lda, ldb elements),
 * C FP32 (row stride ldc), accumulated in FP32 on the tcgen05 tensor cores.
 * k, lda, ldb and k_split must be multiples of 8 and A, B 16-byte aligned;
 * k_split > 0 splits K across CTAs (requires accumulate).  Synchronous on
 * `stream`.  Its bounded waits report through one status word per device,
 * shared by every call: calls that overlap on the GPU (from several host
 * threads, or on several streams) race on that word and may report each
 * other's KIFI_ERR_TIMEOUT; serialise them.  (The proposer's own GEMMs use
 * the status word of their proposer handle.) */
KIFI_API kifi_status kifi_gemm_bf16(const void* a_dev, const void* b_dev, float* c_dev, int m, int n, int k,
                                    int lda, int ldb, int ldc, int k_split, int accumulate, void* stream);

/* No counterpart in the reference.  The proposer's convolution: a 3x3,
 * stride 2, padding 1 convolution of x [batch][height][width][cin] (NHWC
 * BF16, cin 32 or 64) with weights w [cout][kp] (BF16, k = (ky * 3 + kx) *
 * cin + c, cout 64 or 128, kp >= 9 cin) as an implicit GEMM on the tcgen05
 * tensor cores (TMA gathers the input windows; no im2col matrix):
 * out [batch][(height+1)/2][(width+1)/2][cout] = bf16(relu?(conv + bias)),
 * FP32 accumulation, bias FP32 [cout] or NULL.  Synchronous on `stream`;
 * reports through the same status word as kifi_gemm_bf16. */
KIFI_API kifi_status kifi_conv3x3s2_bf16(const void* x_dev, int batch, int height, int width, int cin,
                                         const void* w_dev, int cout, int kp, const float* bias_dev, int relu,
                                         void* out_dev, void* stream);

/* No counterpart in the reference: the learned ICP pose proposer -- a small
 * convolutional network (4 conv 3x3/2 layers 32-64-64-128, global average
 * pool, MLP 128-64-6) mapping two depth frames box-downsampled to 80 x 60 to
 * the 6-DoF twist (rotation vector, translation; camera frame of the first
 * frame) of the second frame's pose relative to the first, used to
 * warm-start ICP.  BF16 weights and activations, FP32 accumulation on the
 * tcgen05 tensor cores (kifi_gemm_bf16), FP32 master weights and Adam.
 * Inputs are NHWC FP16 [batch][60][80][2] (metres, 0 = no depth); batches
 * are multiples of 8 up to max_batch.  Parameters are one FP32 vector of
 * kifi_proposer_param_count entries (layer by layer: weights [out][in],
 * then biases, each padded to a multiple of 8). */
typedef struct kifi_proposer kifi_proposer;
KIFI_API kifi_status kifi_proposer_create(int device, int max_batch, kifi_proposer** out);
KIFI_API kifi_status kifi_proposer_destroy(kifi_proposer* pr);
KIFI_API kifi_status kifi_proposer_param_count(kifi_proposer* pr, size_t* n);
KIFI_API kifi_status kifi_proposer_set_params(kifi_proposer* pr, const float* host, size_t n);
KIFI_API kifi_status kifi_proposer_get_params(kifi_proposer* pr, float* host, size_t n);
/* one network input from two device depth frames (width, height multiples
 * of 80 and 60): per 8x8 block the mean of the non-zero depths, or 0 */
KIFI_API kifi_status kifi_proposer_make_input(kifi_proposer* pr, const void* depth_a_dev,
                                              const void* depth_b_dev, int depth_is_u16, int width,
                                              int height, void* out_fp16_dev);
KIFI_API kifi_status kifi_proposer_set_inputs(kifi_proposer* pr, const void* inputs_fp16_dev, int batch);
KIFI_API kifi_status kifi_proposer_get_inputs(kifi_proposer* pr, void* out_fp16_dev, int batch);
/* forward pass on the inputs set: batch x 6 twists into host memory */
KIFI_API kifi_status kifi_proposer_predict(kifi_proposer* pr, int batch, float* out_twists_host);
/* forward + mean-squared-error loss against targets (device, batch x 6) +
 * backward; the loss and the gradient vector (optional) into host memory */
KIFI_API kifi_status kifi_proposer_gradients(kifi_proposer* pr, const float* targets_dev, int batch,
                                             float* out_loss, float* out_grads_host);
/* kifi_proposer_gradients followed by one Adam step (beta 0.9 / 0.999) */
KIFI_API kifi_status kifi_proposer_train_step(kifi_proposer* pr, const float* targets_dev, int batch,
                                              float lr, float* out_loss);

/* ------------------------------------------------------------ pipeline */

/* Arguments of kifi::Pipeline::Pipeline(cameraParams, volumeResolution,
 * volumeSideLength, truncationMargin) (KinectFission/kifi/Pipeline.h:19-26)
 * plus the tracking and meshing cadence. */
typedef struct kifi_pipeline_desc {
    kifi_camera camera;
    int resolution;
    float side_length_m;
    float truncation_m;
    int icp_iterations;     /* ICP iterations per frame against the previous frame; 0 = off */
    int mesh_every;         /* extract the mesh every N frames (device-resident); 0 = never */
    int mesh_with_indices;  /* Mesh(verts, indices) rather than Mesh(verts) */
    size_t initial_capacity;
    int device;
    int key_bits;           /* as kifi_volume_desc::key_bits */
    int closed_loop;        /* 0: open loop (fuse with the given poses); 1: the reference's
                               tracking path (fuse with the tracked poses, track against the
                               Bin of the model's mesh) -- see kifi_pipeline_integrate */
} kifi_pipeline_desc;

typedef struct kifi_pipeline kifi_pipeline;

KIFI_API kifi_status kifi_pipeline_create(const kifi_pipeline_desc* desc, kifi_pipeline** out);
KIFI_API kifi_status kifi_pipeline_destroy(kifi_pipeline* p);
KIFI_API kifi_volume* kifi_pipeline_volume(kifi_pipeline* p);
KIFI_API kifi_icp* kifi_pipeline_icp(kifi_pipeline* p);

/* kifi::Pipeline::Integrate(rawDepthMap, worldToEye) (Pipeline.h:31-35,
 * Pipeline.cpp:26-56).  Host frame (uint16 mm or float m).
 *
 * Open loop (closed_loop = 0): fuses the frame with its given pose (the
 * reference's live path, :32-35) and, when icp_iterations > 0, also tracks
 * it: ICP against the previous frame's back-projection, with the previous
 * given pose as the guess.  Fusion does not use the tracked pose; frame N+1's
 * fusion overlaps frame N's tracking.
 *
 * Closed loop (closed_loop = 1): the reference's tracking path (:36-55).
 * From the second frame on, ICP aligns the frame against the Bin of the
 * model's mesh starting from the previous tracked pose; the frame is fused
 * with the tracked pose; the volume is meshed (vertices) and binned through
 * EyeToClipRH * worldToEye into a 1024 x 768 target for the next frame.  The
 * first frame's pose is the given one (the reference's constructor fixes
 * it); later given poses are ignored.
 *
 * Every mesh_every frames the output mesh is extracted on the device.
 * Returns with the tracked eye-to-world pose in out_eye_to_world (the given
 * pose's inverse for the first frame or when tracking is off; may be NULL)
 * once the frame's tracking is done and `depth_host` may be reused; the
 * frame's fusion may still be running -- every call that reads the volume
 * (and kifi_pipeline_sync) waits for it and reports its device errors. */
KIFI_API kifi_status kifi_pipeline_integrate(kifi_pipeline* p, const void* depth_host,
                                             int depth_is_u16, const float world_to_eye[16],
                                             float out_eye_to_world[16]);

/* Same with the frame in device memory; asynchronous (the frame must stay
 * valid until the next kifi_pipeline_sync). */
KIFI_API kifi_status kifi_pipeline_integrate_device(kifi_pipeline* p, const void* depth_dev,
                                                    int depth_is_u16,
                                                    const float world_to_eye[16]);

/* Waits for all queued frames and meshes; reports device errors and the
 * last tracked pose (may be NULL). */
KIFI_API kifi_status kifi_pipeline_sync(kifi_pipeline* p, float out_eye_to_world[16]);

/* No counterpart in the reference.  Makes `stream` (a cudaStream_t) wait for
 * all work enqueued so far on the pipeline's streams -- fusion, tracking and
 * meshing -- without blocking the host; e.g. to record one event after a
 * run of frames. */
KIFI_API kifi_status kifi_pipeline_join(kifi_pipeline* p, void* stream);

/* No counterpart in the reference (its stop_watch telemetry).  While the
 * pipeline's volume has profiling on (kifi_volume_set_profiling): the mean
 * device span of an ICP alignment (out_ms[0], per aligned frame) and of an
 * output mesh's counting and emission (out_ms[1], per mesh), with their
 * counts; reading resets them. */
KIFI_API kifi_status kifi_pipeline_stage_times(kifi_pipeline* p, double out_ms[2], int out_counts[2]);

/* No counterpart in the reference.  With graphs on, each frame -- the upload
 * of a page-locked host frame, the fusion launches and the tracking launches
 * on both streams -- runs as one CUDA graph: captured, applied to the
 * instantiated graph with cudaGraphExecUpdate and launched once.  Results
 * are identical to graphs off.  Frames from pageable host memory are uploaded
 * outside the graph.  kifi_pipeline_graph_stats counts instantiations and
 * in-place updates.  Not offered in closed-loop mode (KIFI_ERR_UNSUPPORTED). */
KIFI_API kifi_status kifi_pipeline_set_graphs(kifi_pipeline* p, int on);
KIFI_API kifi_status kifi_pipeline_graph_stats(kifi_pipeline* p, long long* instantiated,
                                               long long* updated);

/* Vertex and index counts of the last output mesh (waits for it). */
KIFI_API kifi_status kifi_pipeline_mesh_counts(kifi_pipeline* p, size_t* n_verts,
                                               size_t* n_indices);
/* Output meshes completed, and how many of them had to be emitted a second
 * time because they outgrew the buffers sized by earlier meshes. */
KIFI_API kifi_status kifi_pipeline_mesh_stats(kifi_pipeline* p, long long* meshes, long long* reemitted);

/* -------------------------------------------------------------- batches */

/* No counterpart in the reference, which runs one kifi::Pipeline at a time.
 * A batch fuses and tracks many independent depth sequences together: one
 * volume and one ICP context per scene (descs[i]: camera, volume, ICP
 * iterations; mesh_every and closed_loop must be 0; one device; every
 * tracked scene uses the same iteration count).  A step takes one device
 * frame (uint16 mm) per scene and enqueues each stage of the path once for
 * all scenes -- splat, sort, merge partition, merge + TSDF update on one
 * stream, ICP begin, the AlignSteps and the next targets' back-projection on
 * another -- each launch sharing its CTAs out among the scenes.  Per scene
 * the results equal kifi_pipeline (open loop) on the same frames. */
typedef struct kifi_batch kifi_batch;
KIFI_API kifi_status kifi_batch_create(const kifi_pipeline_desc* descs, int n, kifi_batch** out);
KIFI_API kifi_status kifi_batch_destroy(kifi_batch* b);
/* one step: depth_dev[i] is scene i's frame (NULL: the scene sits this step
 * out), world_to_eye its pose (16 floats per scene, kifi order).
 * Asynchronous: the frames must stay valid until kifi_batch_sync. */
KIFI_API kifi_status kifi_batch_step_device(kifi_batch* b, const void* const* depth_dev,
                                            const float* world_to_eye);
/* waits for every queued step; reports device errors */
KIFI_API kifi_status kifi_batch_sync(kifi_batch* b);
/* scene i's volume (for kifi_volume_size / export; valid until destroy) */
KIFI_API kifi_volume* kifi_batch_volume(kifi_batch* b, int scene);
/* scene i's last tracked eye-to-world pose (the given one before its first alignment) */
KIFI_API kifi_status kifi_batch_pose(kifi_batch* b, int scene, float out_eye_to_world[16]);
/* the fusion stream (a cudaStream_t): steps end on it */
KIFI_API void* kifi_batch_stream(kifi_batch* b);
/* No counterpart in the reference.  With on != 0 each step's fusion of a
 * key-width group (set-up, splat, digit histograms, digit passes, merge
 * partition, merge + TSDF update of every scene) is one persistent launch of
 * ctas_per_sm CTAs per SM (0: one) whose CTAs walk a device work queue of
 * (stage, scene, chunk) items in stage order; an item first waits, bounded,
 * for its scene's previous stage (KIFI_ERR_TIMEOUT past the bound).  Results
 * equal the launch-per-stage path.  Tracking stays one launch per stage. */
KIFI_API kifi_status kifi_batch_set_persistent(kifi_batch* b, int on, int ctas_per_sm);
/* step timers: while on, every step records its device span (upload of its
 * argument tables to the end of fusion and tracking); kifi_batch_step_times
 * waits for them, returns up to `capacity` spans (ms) and their count, and
 * resets them */
KIFI_API kifi_status kifi_batch_set_profiling(kifi_batch* b, int on);
KIFI_API kifi_status kifi_batch_step_times(kifi_batch* b, float* out_ms, int capacity, int* steps);

#ifdef __cplusplus
}
#endif

#endif /* KIFI_GPU_H */
