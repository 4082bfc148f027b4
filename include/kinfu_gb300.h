/*
 * kinfu_gb300 -- C ABI of the GB300 (sm_103a) KinectFusion per-frame path.
 *
 * Drop-in for the GPU path of PoChang007/Kinect_Fusion_SLAM: the five extern "C"
 * launchers of src/parallel_processing/parallel_processing.h:19-53 and the
 * KinfuPipeline frame loop of src/kinfu_pipeline.{h,cpp}.  Plain pointers and sizes
 * only; no OpenCV, no CUDA or torch types.
 *
 * Conventions (all from the reference):
 *   - millimetres; 4x4 row-major float camera-to-world pose (kinfu_pipeline.h:18);
 *   - 1-based pixel coordinates: the principal point is given in the reference's
 *     convention (cx = 316.625, cy = 256.2318 at kinfu_pipeline.cpp:14-24);
 *   - images are H x W row-major; the predicted-surface planes are world-space mm
 *     with 0 where a ray found no surface (kinfu_pipeline.cpp:195-204);
 *   - volume readback/upload uses the reference's z-fastest order
 *     idx = x*DY*DZ + y*DZ + z (kinfu_pipeline.cpp:53-55) with NaN = unobserved.
 *
 * The library owns all device memory, a CUDA stream and (optionally) captured CUDA
 * graphs per handle; the caller owns every host buffer.  Every call returns a
 * kf_status; kf_last_error() gives the message of the handle's latest failure.
 * A handle must not be used from two threads at once.
 */
#ifndef KINFU_GB300_H
#define KINFU_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int kf_status;
#define KF_OK 0
#define KF_ERR_INVALID_ARGUMENT 1
#define KF_ERR_CUDA 2
#define KF_ERR_OUT_OF_MEMORY 3
#define KF_ERR_STATE 4
#define KF_ERR_IO 5
#define KF_ERR_UNSUPPORTED 6

/* TSDF storage */
#define KF_TSDF_F32 0 /* float value + float weight (reference layout and precision) */
#define KF_TSDF_F16 1 /* half value + half weight pair, 4 bytes per voxel */

/* what an ICP iteration applies when cv::Cholesky would fail (pivot < FLT_EPSILON) */
#define KF_ICP_FAIL_REFERENCE 0 /* as the reference: the raw A^T b is used as the increment */
#define KF_ICP_FAIL_IDENTITY 1  /* skip the increment */

/* summation order of the ICP normal equations (plain FP32 form) */
#define KF_REDUCE_REFERENCE_ORDER 0 /* the reference's 64-pixel trees added in block order: sums
                                       and poses bit-identical to the reference's arithmetic */
#define KF_REDUCE_TREE 1            /* one-pass warp/block/grid tree: faster, sums agree to rounding */

/* 6x6 reduction / solve precision */
#define KF_SOLVE_REFERENCE 0 /* float sums, float-stored Cholesky (cv::Cholesky), float pose */
#define KF_SOLVE_PRECISE 1   /* compensated float sums, FP64 Cholesky and FP64 pose composition */

typedef struct kf_config {
    int height, width;       /* depth image size (480, 640: system_interface.cpp:6-7) */
    float min_depth;         /* mm, inclusive range filter lower bound (300) */
    float max_depth;         /* mm, inclusive upper bound (2000) */
    int dims[3];             /* voxel counts x, y, z (360, 360, 300: kinfu_pipeline.h:46-48) */
    int grid_start[3];       /* integer voxel coordinate of voxel (0,0,0) (-200, -200, -120) */
    float voxel_size;        /* mm (10) */
    float truncated_distance;/* mm (300) */
    float sdf_minimum;       /* mm (-30) */
    float sdf_maximum;       /* mm (300) */
    int icp_levels;          /* 1 = single level as the reference; up to 3 (pyramid) */
    int icp_iterations[3];   /* per level, finest first (10: sensor_pose_estimation.cu:339) */
    float icp_distance;      /* mm correspondence gate (20: sensor_pose_estimation.cu:48) */
    float icp_angle_deg;     /* normal gate in degrees (30: sensor_pose_estimation.cu:69) */
    int icp_fail_mode;       /* KF_ICP_FAIL_* */
    int icp_reduction;       /* KF_REDUCE_* (KF_SOLVE_PRECISE always uses a compensated tree) */
    int solve_mode;          /* KF_SOLVE_* */
    int tsdf_storage;        /* KF_TSDF_* */
    int bilateral;           /* 0 = off as in the reference loop (kinfu_pipeline.cpp:141-145) */
    int bilateral_radius;    /* 3 (kinfu_pipeline.h:58) */
    float sigma_d;           /* 4.5 (kinfu_pipeline.h:61) */
    float sigma_r;           /* 30 (kinfu_pipeline.h:62) */
    int use_graphs;          /* capture the per-frame sequence as CUDA graphs (default 1) */
} kf_config;

typedef struct kf_handle kf_handle;

/* Reference defaults: 480x640, [300, 2000] mm, 360x360x300 @ 10 mm from (-2000,-2000,
 * -1200) mm, truncation 300/-30/300, single-level 10-iteration ICP, FP32. */
void kf_config_default(kf_config* cfg);

/* KinfuPipeline::KinfuPipeline (kinfu_pipeline.cpp:6-65): allocates the device
 * volume (NaN-filled), sets the reference intrinsics and the identity pose. */
kf_status kf_create(const kf_config* cfg, kf_handle** out);
kf_status kf_destroy(kf_handle* h);
const char* kf_last_error(const kf_handle* h);
const char* kf_status_string(kf_status s);
kf_status kf_get_config(const kf_handle* h, kf_config* cfg);

/* intrinsic_matrix (kinfu_pipeline.h:17): fx, fy and the 1-based principal point */
kf_status kf_set_intrinsics(kf_handle* h, float fx, float fy, float cx, float cy);
/* the same with the principal point's convention chosen: one_based != 0 as above;
 * one_based == 0 takes a 0-based (cx, cy), stored as (cx + 1, cy + 1) in float */
kf_status kf_set_intrinsics_ex(kf_handle* h, float fx, float fy, float cx, float cy, int one_based);
kf_status kf_get_intrinsics(const kf_handle* h, float K[9]);
/* extrinsic_matrix (kinfu_pipeline.h:18): 4x4 row-major camera-to-world, mm.  Any
 * matrix is integrated as the reference does; one whose rotation block is more than 2e-4
 * from orthonormal (scaled or sheared) makes integration visit every voxel box (exact,
 * at a dense pass's cost) instead of the boxes its depth tiles can reach. */
kf_status kf_set_pose(kf_handle* h, const float T[16]);
/* Right after a frame call, waits only until that frame's pose is final (the end of its
 * ICP; integration and the ray cast go on in the stream); otherwise waits for all work
 * on the handle's stream. */
kf_status kf_get_pose(kf_handle* h, float T[16]);
/* resets the volume to NaN and the pose to identity; asynchronous on the handle's
 * stream, like the frame calls (the next frame call is kf_initial_processing) */
kf_status kf_reset(kf_handle* h);

/* ---- frame loop (KinfuPipeline) --------------------------------------------------
 * depth: H*W uint16 millimetres (the contents of dep%04d.dat); host pointer, pinned
 * or pageable.  Range filtering to [min_depth, max_depth] happens on the device.  A
 * pinned frame of kf_incoming_frame is copied on a second stream, overlapping the
 * previous frame's work; the caller may reuse the buffer once kf_get_pose or
 * kf_synchronize has returned. */
/* InitialProcessing (kinfu_pipeline.cpp:91-119): integrate at the current pose (first
 * frame semantics) and ray cast the surface prediction */
kf_status kf_initial_processing(kf_handle* h, const uint16_t* depth);
/* IncomingFrameProcessing (kinfu_pipeline.cpp:121-193): vertex/normal map, ICP,
 * integration, ray cast.  Asynchronous on the handle's stream; kf_synchronize (and
 * every call reading images or the volume) waits for it, kf_get_pose for its pose. */
kf_status kf_incoming_frame(kf_handle* h, const uint16_t* depth);
/* one call for both: is_first != 0 is kf_initial_processing, else kf_incoming_frame */
kf_status kf_process_frame(kf_handle* h, const uint16_t* depth, int is_first);
/* same as the two above with device-resident input (a device pointer to H*W uint16),
 * read in the handle's stream order (by kf_incoming_frame_device's graph in place) */
kf_status kf_initial_processing_device(kf_handle* h, const uint16_t* depth_dev);
kf_status kf_incoming_frame_device(kf_handle* h, const uint16_t* depth_dev);
/* reads dep%04d.dat (system_utility.cpp:58-68) from dir into depth (H*W uint16) */
kf_status kf_load_depth_dat(const char* dir, int frame_index, int height, int width, uint16_t* depth);
kf_status kf_synchronize(kf_handle* h);
/* run the handle's work on a caller-owned cudaStream_t (passed as void*); NULL goes
 * back to the handle's own stream.  Captured graphs are launched on whichever stream
 * is current. */
kf_status kf_set_stream(kf_handle* h, void* stream);

/* ray_casting_data->surface_prediction_{x,y,z} and surface_prediction_normal_{x,y,z}
 * (system_utility.h:26-35): six H*W host planes; any pointer may be NULL */
kf_status kf_get_predicted(kf_handle* h, float* x, float* y, float* z, float* nx, float* ny, float* nz);
/* global_tsdf / global_weight_tsdf (kinfu_pipeline.h:24-25) in the reference's order;
 * either pointer may be NULL */
kf_status kf_get_volume(kf_handle* h, float* tsdf, float* weight);
kf_status kf_set_volume(kf_handle* h, const float* tsdf, const float* weight);
/* the range-filtered float depth of the latest frame (depth_image_next) */
kf_status kf_get_depth(kf_handle* h, float* depth);
/* per-iteration ICP log of the latest frame: correspondences, whether the Cholesky
 * factorisation succeeded, and the pose after the iteration (16 floats each); n =
 * number of iterations the arrays hold; any pointer may be NULL */
kf_status kf_get_icp_stats(kf_handle* h, int32_t* ncorr, int32_t* chol_ok, float* poses, int n);

/* ---- stage launchers (parallel_processing.h:19-53), on the handle's device state --
 * Each runs one stage on the depth / pose / prediction the handle holds. */
/* depth input as float (the reference passes cv::Mat CV_32F); no range filter */
kf_status kf_set_depth_f32(kf_handle* h, const float* depth);
/* uint16 input with the range filter (LoadDepthData + GetRangeDepth) */
kf_status kf_set_depth_u16(kf_handle* h, const uint16_t* depth);
/* Calculate_Vertices_And_Normals (raw_vertices.cu:53): outputs may be NULL */
kf_status kf_calculate_vertices_and_normals(kf_handle* h, float* vx, float* vy, float* nx, float* ny, float* nz,
                                            uint8_t* mask);
/* Bilateral_Filtering (bilateral_filtering.cu:49): filters the held depth in place */
kf_status kf_bilateral_filtering(kf_handle* h);
/* Estimate_Sensor_Pose (sensor_pose_estimation.cu:247): ICP from the held vertex map
 * against the held prediction; updates the pose */
kf_status kf_estimate_sensor_pose(kf_handle* h);
/* Projective_TSDF (projective_tsdf.cu:142): integrates the held depth at the pose */
kf_status kf_projective_tsdf(kf_handle* h, int first_tsdf_construct);
/* Ray_Casting (voxel_traversal.cu:426): predicts the surface from the held depth at the
 * pose; hit (may be NULL) receives the z-fastest index of the zero-crossing voxel or -1 */
kf_status kf_ray_casting(kf_handle* h, int32_t* hit);

/* ---- parity hooks --------------------------------------------------------------- */
/* replaces the held prediction (six H*W planes, as kf_get_predicted) */
kf_status kf_set_predicted(kf_handle* h, const float* x, const float* y, const float* z, const float* nx,
                           const float* ny, const float* nz);
/* one ICP association + reduction at the given frame-to-frame F and pose T without
 * updating anything: pair[i] = matched pixel index or -1 (may be NULL), sums27 = the 6
 * entries of A^T b then the 21 of the upper triangle of A^T A, row by row; returns the
 * correspondence count in *ncorr */
kf_status kf_icp_associate(kf_handle* h, const float F[16], const float T[16], int32_t* pair, float* sums27,
                           int32_t* ncorr);
/* the float below which the ray-cast normal is flipped (voxel_traversal.cu:361-369),
 * computed on the device from its own acos at kf_create */
kf_status kf_get_flip_threshold(kf_handle* h, float* c_flip);

/* ---- allocation-free variant ------------------------------------------------------
 * No counterpart in the reference.  One ICP association + normal-equation reduction
 * (as kf_icp_associate, reference summation order) on caller-owned DEVICE buffers,
 * for callers that cannot allocate device memory at this point -- a real-time loop
 * that must not stall on cudaMalloc, or an application that hands out all GPU memory
 * from its own pre-reserved pool.  It allocates nothing: its scratch is a static
 * device array of about 0.55 MB that every GPU loading this library holds until exit.
 *   height * width <= 640 * 480 (307200 pixels), else KF_ERR_UNSUPPORTED;
 *   vmap:   H*W x 4 floats (vx, vy, vz, vertex mask), 16-byte aligned, device;
 *   nmap:   H*W x 4 floats (nx, ny, nz, unused), 16-byte aligned, device;
 *   pred_v, pred_n: the previous ray cast's points / normals, same layout, device;
 *   K, F, T: host 3x3 / 4x4 row-major; dist_mm / angle_deg: the ICP gates (20, 30);
 *   sums28: device, receives the 6 entries of A^T b, the 21 of the upper triangle of
 *           A^T A row by row, and the correspondence count (as a float);
 *   pair:   device H*W int32 (matched pixel index or -1), or NULL;
 *   stream: cudaStream_t passed as void* (NULL = the default stream); it must belong
 *           to the current device, else KF_ERR_INVALID_ARGUMENT.
 * Asynchronous on stream.  A reduction whose bounded wait gave up writes NaN into all
 * 28 entries of sums28.  The first call on each device looks up the scratch array's
 * device address (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  All calls share the scratch array: calls that overlap on the GPU race. */
kf_status kf_icp_associate_noalloc(int height, int width, const float K[9], const float F[16], const float T[16],
                                   const float* vmap, const float* nmap, const float* pred_v, const float* pred_n,
                                   float dist_mm, float angle_deg, float* sums28, int32_t* pair, void* stream);

/* ---- export and checkpoint ------------------------------------------------------
 * kf_export_ply: the latest ray cast's predicted surface as a binary little-endian
 * PLY point cloud (x y z nx ny nz in mm, world frame, red green blue), headless in
 * place of ThreeDViewer::SetUpPointClouds (threeD_viewer.cpp:20-54): a point per pixel
 * whose surface_prediction_z != 0, in pixel order.  colour_bgr: the H*W*3 uint8 BGR
 * image the viewer colours with (system_utility's color_image), host, or NULL to
 * colour each point by its normal.  n_points (may be NULL) receives the point count.
 * Synchronous. */
kf_status kf_export_ply(kf_handle* h, const char* path, const uint8_t* colour_bgr, int* n_points);
/* kf_save_checkpoint / kf_load_checkpoint: the volume, the pose (float and FP64), the
 * intrinsics and the latest prediction, to and from a file, so a run resumes with
 * kf_incoming_frame.  The reference has no counterpart.  Loading needs a handle of the
 * same image size, grid (dims, start, voxel size, truncation) and TSDF storage, else
 * KF_ERR_INVALID_ARGUMENT; a damaged or foreign file gives KF_ERR_IO.  Synchronous. */
kf_status kf_save_checkpoint(kf_handle* h, const char* path);
kf_status kf_load_checkpoint(kf_handle* h, const char* path);

/* ---- differentiation form: trilinear rendering of a TSDF and its adjoint ----------
 * No counterpart in the reference (its ray cast, kf_ray_casting, is not
 * differentiable).  The TSDF is a device float volume in this library's layout
 * (x-fastest, value at voxel centre (index + start + 0.5) * voxel_size, NaN =
 * unobserved), e.g. the handle's FP32 volume.  Per pixel (1-based u, v) the ray
 * o + t R K^-1 [u, v, 1] (t = camera-z depth, mm) is marched from t_near to t_far in
 * steps of `step`, the TSDF sampled trilinearly; the first pair of valid samples with
 * f_a > 0 >= f_b gives depth t* = t_a + step f_a / (f_a - f_b) and the normal
 * grad f / |grad f| at the crossing (world frame).  Pixels without one render 0. */
typedef struct kf_render_desc {
    int height, width;
    float fx, fy, cx, cy; /* the reference's convention: 1-based principal point */
    int dims[3];
    int grid_start[3];
    float voxel_size;
    float t_near, t_far, step; /* mm, camera z */
} kf_render_desc;
/* depth: device H*W floats or NULL; normal: device H*W*3 floats or NULL; T: host 4x4
 * row-major camera-to-world pose.  Asynchronous on stream. */
kf_status kf_render_trilinear(const kf_render_desc* d, const float* tsdf, const float T[16], float* depth,
                              float* normal, void* stream);
/* The adjoint of kf_render_trilinear at (tsdf, T): given dL/d depth (H*W) and dL/d normal
 * (H*W*3) on the device (either may be NULL), ADDS dL/d tsdf into grad_tsdf (device,
 * volume-sized, or NULL) and dL/d xi into grad_pose (device, 6 floats, or NULL), where
 * the pose is perturbed on the left, T(xi) = exp(xi^) T, xi = (omega, tau) in world
 * coordinates.  Recomputes each ray; voxel gradients are added with atomics, so their
 * low bits depend on the order of arrival.  Asynchronous on stream. */
kf_status kf_render_trilinear_backward(const kf_render_desc* d, const float* tsdf, const float T[16],
                                       const float* grad_depth, const float* grad_normal, float* grad_tsdf,
                                       float* grad_pose, void* stream);
/* Gauss-Newton sums of the depth residual r = rendered - measured over the pixels where
 * both are nonzero and |r| <= max_residual (mm; <= 0: no gate -- the gate drops the
 * occlusion edges, as ICP's 20 mm distance test does), with J = d rendered / d xi:
 * sums[0..20] = J^T J (upper triangle row by row), sums[21..26] = J^T r, sums[27] =
 * pixel count, sums[28] = sum r^2 (host, double).  measured_depth: device H*W floats
 * (mm).  Synchronous. */
kf_status kf_render_depth_normal_equations(const kf_render_desc* d, const float* tsdf, const float T[16],
                                           const float* measured_depth, float max_residual, double sums[29],
                                           void* stream);
/* The same under a Huber loss with threshold huber_delta (mm; 0 gives the call above):
 * each pixel's terms are weighted by min(1, huber_delta / |r|) (iteratively reweighted
 * Gauss-Newton), so sums[21..26] = J^T psi(r) with psi(r) = clamp(r, -delta, delta), the
 * loss's gradient; sums[28] = sum of 2 rho(r) (r^2 inside the threshold, 2 delta |r| -
 * delta^2 outside).  Synchronous. */
kf_status kf_render_depth_normal_equations_huber(const kf_render_desc* d, const float* tsdf, const float T[16],
                                                 const float* measured_depth, float max_residual, float huber_delta,
                                                 double sums[29], void* stream);

/* ---- batching form: many scenes, one launch per stage, one graph per frame --------
 * No counterpart in the reference.  A batch owns one kf_handle per scene; the scenes
 * may differ in image size and grid, and share the TSDF storage, the ICP schedule
 * (levels and iterations), the reference-order reduction and the float solve (no
 * bilateral).  Each frame runs every stage as one launch over all scenes (the ray cast
 * is persistent over all scenes' tiles), the whole frame captured as one CUDA graph.
 * Each scene's results are bit-identical to running its handle alone. */
typedef struct kf_batch kf_batch;
kf_status kf_batch_create(const kf_config* configs, int n_scenes, kf_batch** out);
kf_status kf_batch_destroy(kf_batch* b);
/* the scene's handle (owned by the batch; do not destroy): intrinsics, pose, volume,
 * prediction, statistics and checkpoints through the kf_* calls, on the batch's stream */
kf_status kf_batch_scene(kf_batch* b, int scene, kf_handle** out);
/* one frame of every scene: depth[i] = scene i's H_i*W_i uint16 depth in device memory
 * (host array of n_scenes device pointers).  Asynchronous on the batch's stream. */
kf_status kf_batch_initial_processing_device(kf_batch* b, const uint16_t* const* depth);
kf_status kf_batch_incoming_frame_device(kf_batch* b, const uint16_t* const* depth);
kf_status kf_batch_synchronize(kf_batch* b);
/* kernels one kf_batch_incoming_frame_device launches (for all scenes together) */
kf_status kf_batch_kernels_per_frame(kf_batch* b, int* n);
/* Autotuner: times the candidate launch shapes of the idempotent batched stages on the
 * batch's current data (run after a frame) and keeps the fastest: tuning[0] = ICP group
 * pass warps per block (4, 8, 16), [1] = ray-cast tile shape (0: 8x4, 1: 16x2, 2: 4x8
 * pixels per warp), [2] = ray-cast blocks per SM (1..4), [3] = integration z chunk
 * (8, 16, 32; not timed: integration updates the volume).  Synchronous. */
kf_status kf_batch_autotune(kf_batch* b, int tuning[4]);
kf_status kf_batch_set_tuning(kf_batch* b, const int tuning[4]);
/* How integration and the ICP group pass spread the scenes' work: 0 (default) a 2-D
 * grid, one row of blocks per scene (blocks past a smaller scene's extent return at
 * once); 1 a fixed grid over the flattened work of all scenes -- integration boxes taken
 * one at a time from one counter, ICP groups in static strides -- as the ray cast always
 * does.  Results are identical either way.  Synchronous. */
kf_status kf_batch_set_forms(kf_batch* b, int persistent_integration, int persistent_icp);

/* ---- timing --------------------------------------------------------------------- */
/* per-stage device time of the latest kf_incoming_frame (CUDA events, ms):
 * [0] depth+vertex, [1] ICP, [2] integration, [3] ray cast, [4] whole frame.
 * Collected only while enabled (it splits the frame's graph into stages). */
kf_status kf_enable_stage_timing(kf_handle* h, int enable);
kf_status kf_get_stage_times(kf_handle* h, float ms[5]);
/* number of kernels one kf_incoming_frame launches */
kf_status kf_kernels_per_frame(kf_handle* h, int* n);

/* ---- diagnostics (no counterpart in the reference) --------------------------------
 * The polls each of the handle's bounded device waits makes before it gives up, sets
 * the handle's error flag and returns (leaving that ICP iteration's pose unchanged;
 * kf_get_pose then reports KF_ERR_CUDA).  polls >= 0 sets the limit (0: every bounded
 * wait gives up at once -- a host-side way to exercise that error path without a GPU
 * fault); polls < 0 restores the default (2^26 polls, about a second).  Kept across
 * kf_reset.  The reference has no bounded waits (sensor_pose_estimation.cu:399 ignores
 * every failure).  Synchronous. */
kf_status kf_set_wait_limit(kf_handle* h, long long polls);
/* The ICP pose update computes cv::Cholesky's and cv::Mat's double-accumulated results
 * in float-float arithmetic with an exact FP64 fallback.  This runs that code and its
 * FP64 restatement on seeded random 6x6 systems and 4x4 products (blocks x 4 warps x
 * systems_per_warp of each) on the current device and counts: [0] systems, [1] solves
 * that differ in any bit, [2] differing factorisation outcomes, [3] systems that are
 * not positive definite, [4] differing product entries.  Synchronous. */
kf_status kf_selftest_solve(unsigned long long seed, int blocks, int systems_per_warp,
                            unsigned long long counts[5]);
/* The precision form's FP64 solve (fraction-free Gauss-Jordan on [A | b] by a warp
 * pair, a pivot that is not > 0 meaning not positive definite) on n systems given in
 * host memory: A (n x 36 doubles, row-major,
 * symmetric), b (n x 6); writes x (n x 6, untouched where not solved) and ok (n: 1
 * solved, 0 not positive definite).  n <= 1 << 20.  Synchronous. */
kf_status kf_selftest_solve6(const double* A, const double* b, double* x, int* ok, int n);

#ifdef __cplusplus
}
#endif
#endif
