// The handle behind the C ABI's kf_handle (internal to the library): the device-resident
// state of one KinfuPipeline.  Shared by kf_api.cu and the batching form (kf_batch.cu),
// whose scenes are handles of this kind.
#pragma once

#include <string>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "kinfu_gb300.h"
#include "kf_kernels.h"

using kf::Camera;
using kf::Grid;
using kf::IcpParams;
using kf::State;

constexpr int kMaxLevels = kf::kMaxBatchLevels;

struct kf_handle {
    kf_config cfg{};
    Grid grid{};
    Camera cam{};
    IcpParams icp{};
    int device = 0;
    cudaStream_t stream = nullptr;      // stream all work goes to
    cudaStream_t own_stream = nullptr;  // the handle's own stream
    size_t nvox = 0;
    long long skip_from = 0;  // first z-fastest voxel index the reference never integrates

    uint16_t* d_raw = nullptr;
    float* d_depth = nullptr;
    float* d_depth_tmp = nullptr;  // bilateral output
    float4 *d_vmap = nullptr, *d_nmap = nullptr, *d_pv = nullptr, *d_pn = nullptr;
    int32_t* d_hit = nullptr;
    int32_t* d_pair = nullptr;
    float2* d_tab = nullptr;
    long long* d_fixacc = nullptr;  // the precision form's ICP accumulators (icp_fixacc_words)
    float* d_tsdf = nullptr;
    float* d_weight = nullptr;
    __half2* d_vol16 = nullptr;
    State* d_state = nullptr;
    float* d_partials = nullptr;
    int* d_groups = nullptr;  // ICP group flags / compacted group list
    unsigned* d_tiles = nullptr;  // ray-cast tile counter
    unsigned* d_mark = nullptr;   // integration box marks and mark list (2 x integrate_boxes words)
    float* d_mats = nullptr;  // F, T (debug association input) + sums output
    float* d_spatial = nullptr;
    // ICP pyramid: level 0 aliases the buffers above; levels 1.. are half size each
    Camera lcam[kMaxLevels]{};
    float* d_depth_l[kMaxLevels] = {};
    float4 *d_vmap_l[kMaxLevels] = {}, *d_nmap_l[kMaxLevels] = {}, *d_pv_l[kMaxLevels] = {}, *d_pn_l[kMaxLevels] = {};

    uint16_t* h_raw = nullptr;  // pinned staging for pageable host input
    State* h_state = nullptr;   // pinned readback

    cudaGraphExec_t g_incoming = nullptr, g_initial = nullptr;
    bool timing = false;
    cudaEvent_t ev[5] = {};
    float stage_ms[5] = {};
    bool frame_timed = false;
    std::string err;

    // Early pose read-back: a frame call records ev_pose where the frame's pose is final
    // (after the ICP; at once for InitialProcessing), and kf_get_pose right after it
    // copies the pose on aux_stream once that event has passed, while integration and
    // the ray cast still run.  calls counts the API calls on the handle; pose_call is
    // the count after the latest frame call, so any call in between falls back to the
    // full stream synchronisation.
    cudaEvent_t ev_pose = nullptr;
    cudaStream_t aux_stream = nullptr;
    // the side branch that records ev_pose, so that the frame's kernel chain (and its
    // programmatic launches) is not cut by an event node
    cudaStream_t pose_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

    // Pinned host frames are copied on copy_stream into one of two raw buffers (d_raw,
    // d_raw_alt; g_incoming and g_incoming_alt read them), so a frame's copy overlaps the
    // previous frame's integration and ray cast.  ev_raw_free[b] marks the end of the
    // latest stream work that reads buffer b; ev_copied the end of a copy.
    uint16_t* d_raw_alt = nullptr;
    cudaGraphExec_t g_incoming_alt = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied = nullptr, ev_raw_free[2] = {};
    int raw_turn = 0;  // buffer of the latest pinned frame

    // Device-resident frames run g_incoming_dev, whose vertex kernel reads the caller's
    // buffer directly: dev_node is that kernel's node in g_dev_graph and dev_args its
    // argument pointers, the first patched to dev_raw for each frame.
    cudaGraph_t g_dev_graph = nullptr;
    cudaGraphExec_t g_incoming_dev = nullptr;
    cudaGraphNode_t dev_node = nullptr;
    cudaKernelNodeParams dev_params{};
    void* dev_args[16] = {};
    const uint16_t* dev_raw = nullptr;
    mutable unsigned long long calls = 0;
    unsigned long long pose_call = 0;
};
