// Launch wrappers of the kinfu_gb300 kernels (host side; called by kf_api.cu).
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "kf_device.cuh"

namespace kf {

// fill with the reference's NaN (0x7fc00000)
void launch_fill_nan(float* p, size_t n, cudaStream_t s);
void launch_fill_nan_half2(__half2* p, size_t n, cudaStream_t s);

// depth ingest (+ inclusive range filter when raw != nullptr) fused with the
// vertex/normal map of raw_vertices.cu:3-51.  With init_icp, thread 0 also prepares
// the frame's ICP state (T_prev^-1 and F) from st->T.
// the kernel launch_vertex runs on raw input (its first argument is the raw pointer,
// of kVertexKernelArgs arguments), for patching a captured graph's input per frame
constexpr int kVertexKernelArgs = 10;
const void* vertex_raw_kernel_func();
void launch_vertex(const uint16_t* raw, float* depth, float4* vmap, float4* nmap, const Camera& cam, float dmin,
                   float dmax, State* st, bool init_icp, bool compute_normals, cudaStream_t s);

// 7x7 (radius r) bilateral filter of depth into out (bilateral_filtering.cu:3-47); vmap
// (may be nullptr): the vertex map whose z takes the filtered depth
void launch_bilateral(const float* depth, float* out, const float* spatial, int r, float sigma_r, int H, int W,
                      float4* vmap, cudaStream_t s);

// One ICP iteration: association + one-pass reduction + (last block) 6x6 solve and pose
// update.  partials must hold icp_grid_blocks() * kIcpVals floats.
int icp_grid_blocks(int H, int W);
// 64-pixel groups of the reference-order reduction, and the scratch (floats) both
// reductions need; list must hold icp_groups() ints
int icp_groups(int H, int W);
// once per device and image size, outside any stream capture: raises the dynamic
// shared-memory limit of the reduce-and-solve kernel
void icp_prepare(int H, int W);
size_t icp_scratch_floats(int H, int W);
// the precision form's fixed-point accumulators: this many zero-initialised 64-bit words
// (zero again after every launch)
size_t icp_fixacc_words();
// after_pass: the previous launch in the stream is an ICP pass (which writes none of
// vmap, nmap, pv, pn), so the precision form's pass loads vmap and nmap before waiting
// for it
void launch_icp_iteration(const float4* vmap, const float4* nmap, const float4* pv, const float4* pn,
                          const Camera& cam, const IcpParams& prm, State* st, float* partials, int* list,
                          long long* fixacc, bool after_pass, cudaStream_t s);
// Association + reduction only at the given F, T (device pointers to 16 floats each);
// sums_out receives kIcpVals floats (27 sums + count), pair may be nullptr.
void launch_icp_associate(const float4* vmap, const float4* nmap, const float4* pv, const float4* pn,
                          const Camera& cam, const IcpParams& prm, const float* F, const float* T, State* st,
                          float* partials, int* list, long long* fixacc, float* sums_out, int32_t* pair,
                          cudaStream_t s);

// per-pixel integration table + T^-1 and the in-front axis into st
// the integration table (per pixel) and, after its H*W entries, the 8x8-tile depth
// bounds: tab must hold H*W + depth_bound_tiles(H, W) entries
void launch_integrate_prep(const float* depth, float2* tab, const Camera& cam, State* st, cudaStream_t s);
int depth_bound_tiles(int H, int W);
// relative margin of integration's depth-band cull for this camera
float depth_band_eps(const Camera& cam);
// largest |K^-1 (u, v, 1)| over the image (with a margin)
float ray_norm_max(const Camera& cam);
// projective TSDF update (projective_tsdf.cu:5-140) in 32x8x8 voxel boxes, skipping
// the boxes that provably hold no updated voxel: a marking pass over the depth tiles
// marks (mark[box] = 1) every box a tile's pixels can update, a compaction lists the
// marked boxes after the marks and clears the marks, and a persistent pass updates the
// listed boxes; mark holds 2 x integrate_boxes words, zero before the first call;
// skip_from = first z-fastest index the reference's float guard never reaches
void launch_integrate_f32(float* tsdf, float* weight, const float2* tab, const State* st, const Grid& g,
                          const Camera& cam, long long skip_from, bool first, unsigned* mark, cudaStream_t s);
void launch_integrate_f16(__half2* vol, const float2* tab, const State* st, const Grid& g, const Camera& cam,
                          long long skip_from, bool first, unsigned* mark, cudaStream_t s);

// Amanatides-Woo ray cast (voxel_traversal.cu:75-424); hit may be nullptr; tile_counter
// points to two device unsigneds, zero before the first launch, with which the persistent
// kernel hands out ray tiles (the kernel leaves them at zero again)
void launch_raycast_f32(const float* tsdf, const float* depth, float4* pv, float4* pn, int32_t* hit,
                        const Camera& cam, const Grid& g, const State* st, unsigned* tile_counter, cudaStream_t s);
void launch_raycast_f16(const __half2* vol, const float* depth, float4* pv, float4* pn, int32_t* hit,
                        const Camera& cam, const Grid& g, const State* st, unsigned* tile_counter, cudaStream_t s);
// once per device, outside any stream capture: sizes the persistent ray-cast grid
int raycast_blocks();
// the same for the persistent integration pass
int integrate_blocks();

// st->c_flip from the device's own double acos (single thread, once per handle)
void launch_calibrate(State* st, cudaStream_t s);
// ICP pyramid (not in the reference): 2x2 block-averaged depth with a similarity band,
// and the fine level's prediction subsampled at (2i, 2j)
void launch_pyramid_depth(const float* fine, int Wf, float* coarse, int Hc, int Wc, float band, cudaStream_t s);
void launch_pyramid_prediction(const float4* pv_f, const float4* pn_f, int Wf, float4* pv_c, float4* pn_c, int Hc,
                               int Wc, cudaStream_t s);

// ---- the batching form: one launch per stage over a device array of scenes ----------
// max_pixels / max_blocks: the largest scene's count at that level (smaller scenes' extra
// blocks return at once)
void launch_vertex_batch(const SceneDev* scenes, int n_scenes, int max_pixels, int level, bool init_icp,
                         cudaStream_t s);
void launch_pyramid_batch(const SceneDev* scenes, int n_scenes, int max_pixels, int level, cudaStream_t s);
// one ICP iteration of every scene at `level` in the reference summation order: the
// group pass (warps per block: 4, 8 or 16) and one one-warp solve CTA per scene;
// max_groups: the largest scene's 64-pixel groups at that level
void launch_icp_iteration_batch(const SceneDev* scenes, int n_scenes, int max_groups, int level, int warps,
                                cudaStream_t s);
// every scene's integration prep + integration (z chunks of zchunk voxels); max_tiles:
// the largest integrate_tiles() over the scenes
void launch_integrate_batch(const SceneDev* scenes, int n_scenes, int max_pixels, int max_tiles, int zchunk, bool f16,
                            bool first, cudaStream_t s);
int integrate_tiles(const Grid& g, int zchunk);
// integration boxes of the single-scene kernels (the size of the mark array)
int integrate_boxes(const Grid& g);
// every scene's ray cast, persistent over all scenes' tiles; shape 0: 8x4, 1: 16x2,
// 2: 4x8 pixels per warp tile; tile_counter: two device unsigneds, zero between launches
int raycast_tiles(int H, int W, int shape);
void launch_raycast_batch(const SceneDev* scenes, int n_scenes, unsigned total_tiles, bool f16, int shape,
                          int blocks, unsigned* tile_counter, cudaStream_t s);
// the same with the group pass spread over a fixed grid of `blocks` 8-warp blocks (warps
// stride over the flattened groups of all scenes; SceneDev::grp_start must be filled)
void launch_icp_iteration_batch_persistent(const SceneDev* scenes, int n_scenes, int max_groups, int level,
                                           unsigned total_groups, int blocks, cudaStream_t s);
// integration prep + a persistent integration over all scenes' boxes from one counter
// (two device unsigneds, zero between launches; SceneDev::int_start for this zchunk)
void launch_integrate_batch_persistent(const SceneDev* scenes, int n_scenes, int max_pixels, unsigned total_boxes,
                                       int zchunk, bool f16, bool first, int blocks, unsigned* counter, cudaStream_t s);
// the group pass alone (idempotent: what the autotuner times)
void launch_icp_group_batch(const SceneDev* scenes, int n_scenes, int max_groups, int level, int warps, cudaStream_t s);
// packs the predicted points with z != 0 into out (2 float4 per point, unordered) and
// counts them into *count (zero on entry)
void launch_compact_cloud(const float4* pv, const float4* pn, int n, float4* out, unsigned* count, cudaStream_t s);
// identity pose, zeroed ICP bookkeeping and error flag (c_flip kept)
void launch_state_reset(State* st, cudaStream_t s);

// volume layout conversions between the device x-fastest order and the reference's
// z-fastest order
void launch_to_zfast_f32(const float* src, float* dst, const Grid& g, cudaStream_t s);
void launch_from_zfast_f32(const float* src, float* dst, const Grid& g, cudaStream_t s);
void launch_half2_to_zfast(const __half2* src, float* tsdf, float* weight, const Grid& g, cudaStream_t s);
void launch_zfast_to_half2(const float* tsdf, const float* weight, __half2* dst, const Grid& g, cudaStream_t s);

}  // namespace kf
