/*
 * TEST INFRASTRUCTURE -- the CPU oracle.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this library, and only as the checker; the
 * product (kinect_fusion_slam_gb300) never links or calls it.
 *
 * A plain CPU restatement of the reference's per-frame path
 * (PoChang007/Kinect_Fusion_SLAM, src/parallel_processing/*.cu kernel bodies and the
 * host loops of src/kinfu_pipeline.cpp and sensor_pose_estimation.cu), in the
 * reference's own conventions: millimetres, 1-based pixel coordinates, z-fastest
 * voxel order idx = x*DY*DZ + y*DZ + z (kinfu_pipeline.cpp:53-55), NaN for unobserved
 * voxels.  Compiled with -ffp-contract=off so every float operation rounds exactly
 * where the source expression says it does.
 */
#ifndef KF_ORACLE_H
#define KF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kfo_grid {
    int dims[3];      /* voxel counts along x, y, z (voxel_length, voxel_width, voxel_height) */
    int start[3];     /* integer voxel coordinate of voxel (0,0,0): -2000/10, -2000/10, -1200/10 */
    float voxel_size; /* mm */
    float truncated_distance, sdf_minimum, sdf_maximum; /* 300, -30, 300 (kinfu_pipeline.h:51-55) */
} kfo_grid;

/* OpenCV restatements (see ocv_restated.h) exported for the tests */
void kfo_inv3(const float* K, float* Kinv);
int kfo_inv4(const float* T, float* Tinv);
void kfo_matmul4(const float* A, const float* B, float* C);
int kfo_cholesky6(float* A, float* b);

/* thresholds used by the product in place of acos (see tests) */
float kfo_icp_angle_deg(float cos_theta);                 /* sensor_pose_estimation.cu:63-64 */
int kfo_raycast_flip(float cos_theta);                    /* voxel_traversal.cu:361-364 */

/* LoadDepthData + GetRangeDepth: uint16 -> float, zero outside [min, max] inclusive */
void kfo_depth_ingest(const uint16_t* raw, int n, float min_depth, float max_depth, float* out);

/* Calculate_Vertices_And_Normals (raw_vertices.cu:3-51); all outputs fully written */
void kfo_vertex_normal(int H, int W, const float* depth, const float* Kinv,
                       float* vx, float* vy, float* nx, float* ny, float* nz, uint8_t* mask);

/* Projective_TSDF kernel (projective_tsdf.cu:5-140), z-fastest volume */
void kfo_integrate(const kfo_grid* g, int H, int W, const float* depth, const float* K, const float* Kinv,
                   const float* T, const float* Tinv, float* tsdf, float* weight, int first);

/* Voxel_Traversal (voxel_traversal.cu:75-424) with the pinned zero value for the
 * never-assigned XY..ZY; out6 = x,y,z,nx,ny,nz planes (fully written, 0 = miss);
 * hit = z-fastest index of the zero-crossing voxel or -1 */
void kfo_raycast(const kfo_grid* g, int H, int W, const float* depth, const float* Kinv, const float* T,
                 const float* tsdf, float* out6, int32_t* hit);

/* One ICP association pass (sensor_pose_estimation.cu:7-136).  cur6 = vx,vy,vz,nx,ny,nz,
 * pred6 = previous raycast x,y,z,nx,ny,nz.  Writes pair[i] = projected pixel index or -1,
 * and sums42 = the 6 + 36 plane sums in the reference's order (64-wide tree per block,
 * then a serial float sum over blocks, :225-245 and :363-387).  Returns the number of
 * correspondences. */
int kfo_icp_associate(int H, int W, const float* K, const float* F, const float* T,
                      const float* cur6, const uint8_t* mask, const float* pred6,
                      int32_t* pair, float* sums42);

/* Estimate_Sensor_Pose (sensor_pose_estimation.cu:247-470): iters iterations of
 * associate -> reference-order sums -> cv::Cholesky -> small-angle increment -> T <- Inc*T.
 * T is updated in place.  Optional logs: sums_log [iters][42], pose_log [iters][16],
 * ncorr_log [iters], chol_ok_log [iters]. */
/* the per-pixel ICP products (6 a*b then 36 a*a, zero where the pixel is not a
 * correspondence), H*W x 42 floats, for checking reductions */
void kfo_icp_terms(int H, int W, const float* K, const float* F, const float* T, const float* cur6,
                   const uint8_t* mask, const float* pred6, float* terms42);
void kfo_estimate_pose(int H, int W, const float* K, float* T, const float* cur6, const uint8_t* mask,
                       const float* pred6, int iters, float* sums_log, float* pose_log,
                       int32_t* ncorr_log, int32_t* chol_ok_log);

/* Bilateral_Filtering kernel (bilateral_filtering.cu:3-47) with the interior bound
 * tightened to y <= H-1-r, x <= W-1-r so no read leaves the image; pixels outside the
 * interior are 0 as in the reference (whose output buffer starts zeroed).
 * spatial: (2r+1)^2 weights exp(-(dx^2+dy^2)/(2 sigma_d^2)). */
void kfo_bilateral(int H, int W, const float* depth, const float* spatial, int radius, float sigma_r, float* out);

/* ---- whole frame loop (KinfuPipeline, kinfu_pipeline.cpp:6-193) ---- */
typedef struct kfo_pipeline kfo_pipeline;
kfo_pipeline* kfo_create(int H, int W, float min_depth, float max_depth, const kfo_grid* g, const float* K,
                         int icp_iters);
void kfo_destroy(kfo_pipeline* p);
/* InitialProcessing (kinfu_pipeline.cpp:91-119) */
void kfo_initial(kfo_pipeline* p, const uint16_t* raw);
/* IncomingFrameProcessing (kinfu_pipeline.cpp:121-193), bilateral disabled as in the
 * reference unless kfo_set_bilateral enabled it */
void kfo_incoming(kfo_pipeline* p, const uint16_t* raw);
/* the bilateral stage at the reference's commented-out call site (kinfu_pipeline.cpp:141-145) */
void kfo_set_bilateral(kfo_pipeline* p, int enable, int radius, float sigma_d, float sigma_r);
/* kfo_incoming with the bilateral stage's output given (H*W floats) instead of computed */
void kfo_incoming_filtered(kfo_pipeline* p, const uint16_t* raw, const float* filtered);
/* ICP pyramid (not in the reference): levels 1..3, iterations per level finest first,
 * depth-similarity band of the block averaging (mm) */
void kfo_set_pyramid(kfo_pipeline* p, int levels, const int* iters, float band);
void kfo_pyramid_depth(int Hf, int Wf, const float* fine, float band, float* coarse);
void kfo_level_intrinsics(const float* K, int l, float* Kl);
void kfo_get_pose(const kfo_pipeline* p, float* T);
void kfo_set_pose(kfo_pipeline* p, const float* T);
/* 6 planes HxW (x,y,z,nx,ny,nz), and the hit plane */
void kfo_get_prediction(const kfo_pipeline* p, float* out6, int32_t* hit);
void kfo_get_volume(const kfo_pipeline* p, float* tsdf, float* weight);
void kfo_get_depth(const kfo_pipeline* p, float* depth);
/* cur6 = vx,vy,vz(depth),nx,ny,nz of the latest incoming frame, mask */
void kfo_get_vertex_map(const kfo_pipeline* p, float* cur6, uint8_t* mask);

int kfo_num_threads(void);

/* ---- the FP64 oracle (kf_oracle64.cpp): the same frame loop with every quantity in
 * double and a double Cholesky solve; the yardstick of the precision form ---- */
typedef struct kfo64_pipeline kfo64_pipeline;
kfo64_pipeline* kfo64_create(int H, int W, double min_depth, double max_depth, const kfo_grid* g, const double* K,
                             int icp_iters);
void kfo64_destroy(kfo64_pipeline* p);
void kfo64_initial(kfo64_pipeline* p, const uint16_t* raw);
void kfo64_incoming(kfo64_pipeline* p, const uint16_t* raw);
void kfo64_get_pose(const kfo64_pipeline* p, double* T);
void kfo64_set_pose(kfo64_pipeline* p, const double* T);
/* single stages at the current pose */
void kfo64_integrate_frame(kfo64_pipeline* p, const uint16_t* raw, int first);
void kfo64_raycast_frame(kfo64_pipeline* p);
/* world-space predicted points and normals, 6 planes of H*W */
void kfo64_get_prediction(const kfo64_pipeline* p, double* out6);
/* the volume rounded to float, z-fastest reference order */
void kfo64_get_volume(const kfo64_pipeline* p, float* tsdf, float* weight);

#ifdef __cplusplus
}
#endif
#endif
