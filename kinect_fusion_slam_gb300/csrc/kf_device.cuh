// Device-side types and helpers shared by the kinfu_gb300 kernels.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "kf_divmagic.h"
#include "kf_math.cuh"

namespace kf {

constexpr int kMaxIcpIters = 64;
// per-block ICP partial: 6 sums of a*b, 21 of the upper triangle of a a^T, count
constexpr int kIcpVals = 28;

// The voxel grid.  Device layout is x-fastest: lin = (z*dy + y)*dx + x; the
// reference's z-fastest index is (x*dy + y)*dz + z (kinfu_pipeline.cpp:53-55).
struct Grid {
    int dx, dy, dz;
    int sx, sy, sz;  // integer voxel coordinate of voxel (0,0,0)
    float vd;        // voxel size, mm
    float trunc, sdf_min, sdf_max;
    DivMagic qdx, qdy;  // division by dx and by dy (decoding linear indices)
};

struct Camera {
    int H, W;
    float K[9], Ki[9];
};

struct IcpParams {
    float dist;       // mm
    float angle_deg;  // degrees
    int fail_mode;        // 0 reference (raw b), 1 identity
    int precise;          // compensated sums + FP64 solve
    int reference_order;  // sums in the reference's order (bit-identical to it)
    // the precision form's association gates in the form it evaluates them: dist^2
    // (negative: nothing passes) and cos(angle)
    float dist2;
    float cos_angle;
};

// Per-handle device state, updated by the kernels so that a whole frame runs without
// host round trips.
struct State {
    float T[16];          // extrinsic_matrix: camera-to-world pose
    int error;            // set by a kernel whose bounded wait gave up (read with T)
    float Tprev_inv[16];  // inverse of the pose at the start of the frame's ICP
    float F[16];          // Tprev_inv * T, the frame-to-frame transform of the iteration
    float Tinv[16];       // inverse of the pose used by integration
    float Tinv_src[16];   // the pose Tinv was computed from
    float axis[3];        // "in front of the camera" direction (projective_tsdf.cu:57-71)
    float c_flip;         // ray-cast normal flip threshold (voxel_traversal.cu:361-369)
    unsigned mark_count;  // boxes on integration's mark list (reset by integrate_prep)
    unsigned mark_near;   // some tile's depth band reaches near the camera (reset likewise)
    unsigned mark_all;    // some tile's band has no finite depth bound: every box is listed (likewise)
    double Td[16];        // FP64 pose (precise solve mode)
    unsigned ticket;      // last-block election counter of the ICP reduction
    int iter;             // ICP iterations done in the current frame
    int32_t ncorr[kMaxIcpIters];
    int32_t chol_ok[kMaxIcpIters];
    float Tlog[kMaxIcpIters][16];  // pose after each iteration
    float sums[kIcpVals];  // sums of the most recent ICP iteration
    unsigned fix_bad;      // precision form: sums whose block values could not be accumulated
    // polls a bounded wait makes before it gives up and sets error (kept across resets;
    // kDefaultWaitLimit unless a test lowers it to exercise the error path)
    long long wait_limit;
};

// about 1 s of polling: a copy or a peer that has not arrived by then is reported
constexpr long long kDefaultWaitLimit = 1LL << 26;

// One scene of a batch (the batching form): the device buffers and parameters its
// kernels need.  A batched launch covers every scene; blockIdx.y (or a flattened tile
// index) picks the scene from a device array of these.  Level 0 aliases a handle's own
// buffers, levels 1.. its ICP pyramid.
constexpr int kMaxBatchLevels = 3;
struct SceneDev {
    Camera cam[kMaxBatchLevels];
    Grid grid;
    IcpParams icp;
    const uint16_t* raw;  // this frame's depth, device
    float* depth[kMaxBatchLevels];
    float4* vmap[kMaxBatchLevels];
    float4* nmap[kMaxBatchLevels];
    float4* pv[kMaxBatchLevels];
    float4* pn[kMaxBatchLevels];
    float2* tab;
    float* tsdf;
    float* weight;
    __half2* vol16;
    State* st;
    float* partials;
    int* groups;
    int32_t* hit;
    long long skip_from;
    float dmin, dmax, band;
    int tile_start[3];  // first ray-cast tile of this scene for tile shapes 8x4, 16x2, 4x8
    float depth_eps;    // integration's depth-band cull margin (depth_band_eps)
    float lam_max;      // ray_norm_max
    // the scene's first integration box and first ICP group (per pyramid level) in the
    // batch's flattened lists, for the launches that spread all scenes' work over the GPU
    int int_start;
    int grp_start[kMaxBatchLevels];
};

// voxel-centre coordinate, kinfu_pipeline.cpp:53-55: x * voxel_distance + voxel_distance / 2
__device__ __forceinline__ float centre(int index, int start, float vd)
{
    return (float)(index + start) * vd + vd / 2.f;
}

// rows 0..2 of a 4x4 row-major transform applied to a point, ((m0 x + m1 y) + m2 z) + m3
__device__ __forceinline__ float3 xform(const float* m, float3 p)
{
    return make_float3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                       m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}

__device__ __forceinline__ float3 mul3(const float* m, float3 p)
{
    return make_float3(m[0] * p.x + m[1] * p.y + m[2] * p.z, m[3] * p.x + m[4] * p.y + m[5] * p.z,
                       m[6] * p.x + m[7] * p.y + m[8] * p.z);
}

// Get_Normalized, cuda_functions.cuh:1-10
__device__ __forceinline__ float3 normalized(float3 v)
{
    const float r = 1 / sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return make_float3(v.x * r, v.y * r, v.z * r);
}

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

}  // namespace kf
