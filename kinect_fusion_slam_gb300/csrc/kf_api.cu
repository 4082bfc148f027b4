// C ABI of the kinfu_gb300 library (include/kinfu_gb300.h).
//
// A handle owns the device-resident state of one KinfuPipeline: the volume, the
// depth / vertex / prediction images, the pose and ICP scratch in a State block, a
// CUDA stream and, optionally, the per-frame kernel sequence captured as CUDA graphs.
// The pose never leaves the device during a frame: every kernel reads it from, and
// the ICP's last block writes it to, the State block.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "kinfu_gb300.h"
#include "kf_kernels.h"
#include "kf_handle.h"

using namespace kf;


namespace {

kf_status fail(kf_handle* h, kf_status s, const std::string& msg)
{
    if (h) h->err = msg;
    return s;
}

#define KF_CUDA(h, call)                                                                                  \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            return fail((h), e_ == cudaErrorMemoryAllocation ? KF_ERR_OUT_OF_MEMORY : KF_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                              \
        }                                                                                                 \
    } while (0)

#define KF_CHECK_LAUNCH(h) KF_CUDA(h, cudaGetLastError())

template <class T>
T* field_ptr(State* st, size_t offset)
{
    return reinterpret_cast<T*>(reinterpret_cast<char*>(st) + offset);
}

void destroy_graphs(kf_handle* h)
{
    if (h->g_incoming) cudaGraphExecDestroy(h->g_incoming);
    if (h->g_incoming_alt) cudaGraphExecDestroy(h->g_incoming_alt);
    if (h->g_initial) cudaGraphExecDestroy(h->g_initial);
    if (h->g_incoming_dev) cudaGraphExecDestroy(h->g_incoming_dev);
    if (h->g_dev_graph) cudaGraphDestroy(h->g_dev_graph);
    h->g_incoming = h->g_incoming_alt = h->g_initial = h->g_incoming_dev = nullptr;
    h->g_dev_graph = nullptr;
    h->dev_node = nullptr;
}

bool validate(const kf_config* c, std::string& why)
{
    if (c->height < 2 || c->width < 2 || (long long)c->height * c->width > (1LL << 26)) {
        why = "image size out of range";
        return false;
    }
    for (int k = 0; k < 3; ++k)
        if (c->dims[k] < 3 || c->dims[k] > 4096) {
            why = "grid dimensions out of range";
            return false;
        }
    if (c->icp_reduction == KF_REDUCE_REFERENCE_ORDER && (long long)c->height * c->width > 32768LL * 64) {
        why = "the reference-order ICP reduction supports up to 2097152 pixels";
        return false;
    }
    if ((double)c->dims[0] * c->dims[1] * c->dims[2] > 2147483647.0) {
        why = "grid has more than 2^31-1 voxels (the reference indexes voxels with int)";
        return false;
    }
    if (!(c->voxel_size > 0) || !(c->truncated_distance > 0)) {
        why = "voxel_size and truncated_distance must be positive";
        return false;
    }
    if (c->icp_levels < 1 || c->icp_levels > kMaxLevels) {
        why = "icp_levels must be 1 (the reference), 2 or 3";
        return false;
    }
    int total = 0;
    for (int l = 0; l < c->icp_levels; ++l) {
        if (c->icp_iterations[l] < 0 || c->icp_iterations[l] > kMaxIcpIters) {
            why = "icp_iterations out of range [0, 64]";
            return false;
        }
        total += c->icp_iterations[l];
    }
    if (total > kMaxIcpIters) {
        why = "more than 64 ICP iterations per frame";
        return false;
    }
    if (c->icp_levels > 1) {
        const int f = 1 << (c->icp_levels - 1);
        if (c->height % f || c->width % f || c->height / f < 8 || c->width / f < 8) {
            why = "the pyramid needs height and width divisible by 2^(icp_levels-1), coarsest level >= 8x8";
            return false;
        }
    }
    if (c->icp_reduction != KF_REDUCE_REFERENCE_ORDER && c->icp_reduction != KF_REDUCE_TREE) {
        why = "unknown icp_reduction";
        return false;
    }
    if (c->tsdf_storage != KF_TSDF_F32 && c->tsdf_storage != KF_TSDF_F16) {
        why = "unknown tsdf_storage";
        return false;
    }
    if (c->bilateral_radius < 1 || c->bilateral_radius > 7) {
        why = "bilateral_radius must be in [1, 7]";
        return false;
    }
    return true;
}

// smallest z-fastest index i with (float)i >= (float)DX * (float)DY * (float)DZ: the
// reference kernel's guard (projective_tsdf.cu:14) returns for these threads
long long float_guard_start(const int* d)
{
    const float nf = (float)d[0] * (float)d[1] * (float)d[2];
    long long n = (long long)d[0] * d[1] * d[2];
    long long i = n;
    while (i > 0 && (float)(i - 1) >= nf) --i;
    return i;
}

kf_status upload_raw(kf_handle* h, const uint16_t* depth)
{
    const size_t bytes = sizeof(uint16_t) * h->cam.H * h->cam.W;
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, depth) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    if (pinned) {
        KF_CUDA(h, cudaMemcpyAsync(h->d_raw, depth, bytes, cudaMemcpyHostToDevice, h->stream));
    } else {
        // the staging buffer may still feed an earlier copy
        KF_CUDA(h, cudaStreamSynchronize(h->stream));
        std::memcpy(h->h_raw, depth, bytes);
        KF_CUDA(h, cudaMemcpyAsync(h->d_raw, h->h_raw, bytes, cudaMemcpyHostToDevice, h->stream));
    }
    return KF_OK;
}

bool is_pinned(const void* p)
{
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, p) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return pinned;
}

// the stream work enqueued so far is the latest to read buffer b
void raw_used(kf_handle* h, int b) { cudaEventRecord(h->ev_raw_free[b], h->stream); }

// A pinned host frame's copy into the other raw buffer on copy_stream, after the latest
// work that read that buffer (the frame before the previous one, normally long done) and
// concurrent with the previous frame's work; the frame's stream waits for the copy.
// (The host wrote the frame before the call, so the copy needs no stream order.)
// Returns the buffer.
kf_status upload_raw_async(kf_handle* h, const uint16_t* depth, cudaMemcpyKind kind, int& buf)
{
    const size_t bytes = sizeof(uint16_t) * h->cam.H * h->cam.W;
    buf = h->raw_turn ^ 1;
    uint16_t* dst = buf ? h->d_raw_alt : h->d_raw;
    KF_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->ev_raw_free[buf], 0));
    KF_CUDA(h, cudaMemcpyAsync(dst, depth, bytes, kind, h->copy_stream));
    KF_CUDA(h, cudaEventRecord(h->ev_copied, h->copy_stream));
    KF_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_copied, 0));
    h->raw_turn = buf;
    return KF_OK;
}

// ---- stage enqueuers (no synchronisation) ----
void enq_ingest(kf_handle* h, const uint16_t* raw, bool init_icp, bool normals)
{
    launch_vertex(raw, h->d_depth, h->d_vmap, h->d_nmap, h->cam, h->cfg.min_depth, h->cfg.max_depth, h->d_state,
                  init_icp, normals, h->stream);
}

void enq_bilateral(kf_handle* h)
{
    launch_bilateral(h->d_depth, h->d_depth_tmp, h->d_spatial, h->cfg.bilateral_radius, h->cfg.sigma_r, h->cam.H,
                     h->cam.W, h->d_vmap, h->stream);
    cudaMemcpyAsync(h->d_depth, h->d_depth_tmp, sizeof(float) * h->cam.H * h->cam.W, cudaMemcpyDeviceToDevice,
                    h->stream);
}

// ICP of one frame.  With a pyramid (not in the reference, which tracks at full
// resolution only), the coarser levels' depth, vertex/normal maps and previous-frame
// predictions are derived first, then the iterations run coarsest level first; the pose
// carries over between levels.
void enq_icp(kf_handle* h)
{
    const int L = h->cfg.icp_levels;
    for (int l = 1; l < L; ++l) {
        const Camera& f = h->lcam[l - 1];
        const Camera& c = h->lcam[l];
        launch_pyramid_depth(h->d_depth_l[l - 1], f.W, h->d_depth_l[l], c.H, c.W, 3.0f * h->cfg.sigma_r, h->stream);
        launch_vertex(nullptr, h->d_depth_l[l], h->d_vmap_l[l], h->d_nmap_l[l], c, h->cfg.min_depth, h->cfg.max_depth,
                      h->d_state, false, true, h->stream);
        launch_pyramid_prediction(h->d_pv_l[l - 1], h->d_pn_l[l - 1], f.W, h->d_pv_l[l], h->d_pn_l[l], c.H, c.W,
                                  h->stream);
    }
    bool after_pass = false;  // the previous launch in the stream is an ICP pass
    for (int l = L - 1; l >= 0; --l)
        for (int it = 0; it < h->cfg.icp_iterations[l]; ++it) {
            launch_icp_iteration(h->d_vmap_l[l], h->d_nmap_l[l], h->d_pv_l[l], h->d_pn_l[l], h->lcam[l], h->icp,
                                 h->d_state, h->d_partials, h->d_groups, h->d_fixacc, after_pass, h->stream);
            after_pass = true;
        }
}

void enq_integrate(kf_handle* h, bool first)
{
    launch_integrate_prep(h->d_depth, h->d_tab, h->cam, h->d_state, h->stream);
    if (h->d_vol16)
        launch_integrate_f16(h->d_vol16, h->d_tab, h->d_state, h->grid, h->cam, h->skip_from, first, h->d_mark,
                             h->stream);
    else
        launch_integrate_f32(h->d_tsdf, h->d_weight, h->d_tab, h->d_state, h->grid, h->cam, h->skip_from, first,
                             h->d_mark, h->stream);
}

void enq_raycast(kf_handle* h, int32_t* hit)
{
    if (h->d_vol16)
        launch_raycast_f16(h->d_vol16, h->d_depth, h->d_pv, h->d_pn, hit, h->cam, h->grid, h->d_state, h->d_tiles,
                           h->stream);
    else
        launch_raycast_f32(h->d_tsdf, h->d_depth, h->d_pv, h->d_pn, hit, h->cam, h->grid, h->d_state, h->d_tiles,
                           h->stream);
}

// stage timing event k; inside a stream capture the record must be an external
// event node to fire when the graph is replayed
void stamp(kf_handle* h, int k)
{
    if (!h->timing) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(h->stream, &cs);
    if (cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(h->ev[k], h->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(h->ev[k], h->stream);
}

// IncomingFrameProcessing after the depth upload (kinfu_pipeline.cpp:128-188).  The
// bilateral call site the reference leaves commented out sits after the vertex map
// (kinfu_pipeline.cpp:141-145): when enabled here it filters the depth that ICP,
// integration and ray casting use, in the same place.
// ev_pose where the frame's pose is final: recorded on a side branch forked from the
// frame's stream at this point (an external event node when captured) and joined back
// by join_pose at the end of the frame
void mark_pose(kf_handle* h)
{
    cudaEventRecord(h->ev_fork, h->stream);
    cudaStreamWaitEvent(h->pose_stream, h->ev_fork, 0);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(h->stream, &cs);
    if (cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(h->ev_pose, h->pose_stream, cudaEventRecordExternal);
    else
        cudaEventRecord(h->ev_pose, h->pose_stream);
    cudaEventRecord(h->ev_join, h->pose_stream);
}

void join_pose(kf_handle* h) { cudaStreamWaitEvent(h->stream, h->ev_join, 0); }

void enq_incoming(kf_handle* h, const uint16_t* raw)
{
    stamp(h, 0);
    enq_ingest(h, raw, true, true);
    if (h->cfg.bilateral) enq_bilateral(h);
    stamp(h, 1);
    enq_icp(h);
    mark_pose(h);
    stamp(h, 2);
    enq_integrate(h, false);
    stamp(h, 3);
    enq_raycast(h, h->d_hit);
    stamp(h, 4);
    join_pose(h);
}

// InitialProcessing after the depth upload (kinfu_pipeline.cpp:93-115)
void enq_initial(kf_handle* h, const uint16_t* raw)
{
    mark_pose(h);  // InitialProcessing keeps the pose
    enq_ingest(h, raw, false, true);
    enq_integrate(h, true);
    enq_raycast(h, h->d_hit);
    join_pose(h);
}

kf_status run_captured(kf_handle* h, cudaGraphExec_t& exec, bool incoming, const uint16_t* raw)
{
    if (!h->cfg.use_graphs) {
        if (incoming)
            enq_incoming(h, raw);
        else
            enq_initial(h, raw);
        KF_CHECK_LAUNCH(h);
        return KF_OK;
    }
    if (!exec) {
        cudaGraph_t graph = nullptr;
        KF_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        if (incoming)
            enq_incoming(h, raw);
        else
            enq_initial(h, raw);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(h, KF_ERR_CUDA,
                        std::string("graph capture failed: ") + cudaGetErrorString(le != cudaSuccess ? le : ce));
        }
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            exec = nullptr;
            return fail(h, KF_ERR_CUDA, std::string("graph instantiate failed: ") + cudaGetErrorString(ie));
        }
    }
    KF_CUDA(h, cudaGraphLaunch(exec, h->stream));
    return KF_OK;
}

kf_status read_state(kf_handle* h)
{
    KF_CUDA(h, cudaMemcpyAsync(h->h_state, h->d_state, sizeof(State), cudaMemcpyDeviceToHost, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

void set_camera(kf_handle* h, float fx, float fy, float cx, float cy)
{
    float K[9] = {fx, 0.0f, cx, 0.0f, fy, cy, 0.0f, 0.0f, 1.0f};
    std::memcpy(h->cam.K, K, sizeof(K));
    inv3(h->cam.K, h->cam.Ki);
    h->lcam[0] = h->cam;
    // level l halves the image l times: focal lengths / 2^l, and the 1-based principal
    // point maps as (c - 1/2) / 2^l + 1/2 (pixel centres of the 2x2 blocks)
    for (int l = 1; l < kMaxLevels; ++l) {
        const float s = 1.0f / (float)(1 << l);
        Camera& c = h->lcam[l];
        c.H = h->cam.H >> l;
        c.W = h->cam.W >> l;
        const float Kl[9] = {fx * s, 0.0f, (cx - 0.5f) * s + 0.5f, 0.0f, fy * s, (cy - 0.5f) * s + 0.5f,
                             0.0f, 0.0f, 1.0f};
        std::memcpy(c.K, Kl, sizeof(Kl));
        inv3(c.K, c.Ki);
    }
}

template <class T>
kf_status dalloc(kf_handle* h, T** p, size_t count)
{
    KF_CUDA(h, cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)));
    return KF_OK;
}

#define KF_TRY(expr)                      \
    do {                                  \
        kf_status s_ = (expr);            \
        if (s_ != KF_OK) return s_;       \
    } while (0)

#define KF_HANDLE(h)                                    \
    do {                                                \
        if (!(h)) return KF_ERR_INVALID_ARGUMENT;       \
        ++(h)->calls;                                   \
        cudaSetDevice((h)->device);                     \
    } while (0)

kf_status allocate(kf_handle* h)
{
    const size_t HW = (size_t)h->cam.H * h->cam.W;
    KF_TRY(dalloc(h, &h->d_raw, HW));
    KF_TRY(dalloc(h, &h->d_raw_alt, HW));
    KF_TRY(dalloc(h, &h->d_depth, HW));
    KF_TRY(dalloc(h, &h->d_depth_tmp, HW));
    KF_TRY(dalloc(h, &h->d_vmap, HW));
    KF_TRY(dalloc(h, &h->d_nmap, HW));
    KF_TRY(dalloc(h, &h->d_pv, HW));
    KF_TRY(dalloc(h, &h->d_pn, HW));
    KF_TRY(dalloc(h, &h->d_hit, HW));
    KF_TRY(dalloc(h, &h->d_pair, HW));
    KF_TRY(dalloc(h, &h->d_tab, HW + depth_bound_tiles(h->cam.H, h->cam.W)));
    KF_TRY(dalloc(h, &h->d_state, 1));
    KF_TRY(dalloc(h, &h->d_partials, icp_scratch_floats(h->cam.H, h->cam.W)));
    KF_TRY(dalloc(h, &h->d_fixacc, icp_fixacc_words()));
    KF_CUDA(h, cudaMemsetAsync(h->d_fixacc, 0, icp_fixacc_words() * sizeof(long long), h->stream));
    KF_TRY(dalloc(h, &h->d_groups, (size_t)icp_groups(h->cam.H, h->cam.W)));
    KF_TRY(dalloc(h, &h->d_tiles, 2));
    KF_CUDA(h, cudaMemset(h->d_tiles, 0, 2 * sizeof(unsigned)));
    // box marks, then the list of marked boxes
    KF_TRY(dalloc(h, &h->d_mark, 2 * (size_t)integrate_boxes(h->grid)));
    KF_CUDA(h, cudaMemset(h->d_mark, 0, 2 * sizeof(unsigned) * (size_t)integrate_boxes(h->grid)));
    KF_TRY(dalloc(h, &h->d_mats, 64));
    KF_TRY(dalloc(h, &h->d_spatial, 15 * 15));
    h->d_depth_l[0] = h->d_depth;
    h->d_vmap_l[0] = h->d_vmap;
    h->d_nmap_l[0] = h->d_nmap;
    h->d_pv_l[0] = h->d_pv;
    h->d_pn_l[0] = h->d_pn;
    for (int l = 1; l < h->cfg.icp_levels; ++l) {
        const size_t n = HW >> (2 * l);
        KF_TRY(dalloc(h, &h->d_depth_l[l], n));
        KF_TRY(dalloc(h, &h->d_vmap_l[l], n));
        KF_TRY(dalloc(h, &h->d_nmap_l[l], n));
        KF_TRY(dalloc(h, &h->d_pv_l[l], n));
        KF_TRY(dalloc(h, &h->d_pn_l[l], n));
    }
    if (h->cfg.tsdf_storage == KF_TSDF_F16) {
        KF_TRY(dalloc(h, &h->d_vol16, h->nvox));
    } else {
        KF_TRY(dalloc(h, &h->d_tsdf, h->nvox));
        KF_TRY(dalloc(h, &h->d_weight, h->nvox));
    }
    KF_CUDA(h, cudaMallocHost((void**)&h->h_raw, sizeof(uint16_t) * HW));
    KF_CUDA(h, cudaMallocHost((void**)&h->h_state, sizeof(State)));
    for (auto& e : h->ev) KF_CUDA(h, cudaEventCreate(&e));
    KF_CUDA(h, cudaEventCreateWithFlags(&h->ev_pose, cudaEventDisableTiming));
    KF_CUDA(h, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    KF_CUDA(h, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    KF_CUDA(h, cudaStreamCreateWithFlags(&h->aux_stream, cudaStreamNonBlocking));
    KF_CUDA(h, cudaStreamCreateWithFlags(&h->pose_stream, cudaStreamNonBlocking));
    KF_CUDA(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    KF_CUDA(h, cudaEventCreateWithFlags(&h->ev_copied, cudaEventDisableTiming));
    for (auto& e : h->ev_raw_free) KF_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return KF_OK;
}

// volume to NaN, images to "no data"; stream-ordered, no host synchronisation
kf_status enqueue_clear(kf_handle* h)
{
    const size_t HW = (size_t)h->cam.H * h->cam.W;
    if (h->d_vol16)
        launch_fill_nan_half2(h->d_vol16, h->nvox, h->stream);
    else {
        launch_fill_nan(h->d_tsdf, h->nvox, h->stream);
        launch_fill_nan(h->d_weight, h->nvox, h->stream);
    }
    KF_CHECK_LAUNCH(h);
    KF_CUDA(h, cudaMemsetAsync(h->d_depth, 0, sizeof(float) * HW, h->stream));
    KF_CUDA(h, cudaMemsetAsync(h->d_vmap, 0, sizeof(float4) * HW, h->stream));
    KF_CUDA(h, cudaMemsetAsync(h->d_nmap, 0, sizeof(float4) * HW, h->stream));
    KF_CUDA(h, cudaMemsetAsync(h->d_pv, 0, sizeof(float4) * HW, h->stream));
    KF_CUDA(h, cudaMemsetAsync(h->d_pn, 0, sizeof(float4) * HW, h->stream));
    KF_CUDA(h, cudaMemsetAsync(h->d_hit, 0xff, sizeof(int32_t) * HW, h->stream));
    return KF_OK;
}

// first initialisation at kf_create: clear, identity pose, calibrated c_flip
kf_status reset_state(kf_handle* h)
{
    KF_TRY(enqueue_clear(h));
    std::memset(h->h_state, 0, sizeof(State));
    h->h_state->wait_limit = kf::kDefaultWaitLimit;
    for (int k = 0; k < 16; ++k) {
        h->h_state->T[k] = (k % 5 == 0) ? 1.f : 0.f;
        h->h_state->Td[k] = (k % 5 == 0) ? 1.0 : 0.0;
    }
    KF_CUDA(h, cudaMemcpyAsync(h->d_state, h->h_state, sizeof(State), cudaMemcpyHostToDevice, h->stream));
    launch_calibrate(h->d_state, h->stream);
    KF_CHECK_LAUNCH(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

void free_all(kf_handle* h)
{
    destroy_graphs(h);
    void* dev[] = {h->d_raw, h->d_raw_alt, h->d_depth, h->d_depth_tmp, h->d_vmap, h->d_nmap, h->d_pv, h->d_pn, h->d_hit,
                   h->d_pair, h->d_tab, h->d_tsdf, h->d_weight, h->d_vol16, h->d_state, h->d_partials, h->d_groups,
                   h->d_fixacc,
                   h->d_tiles, h->d_mark, h->d_mats,
                   h->d_spatial};
    for (void* p : dev)
        if (p) cudaFree(p);
    for (int l = 1; l < kMaxLevels; ++l) {
        void* lv[] = {h->d_depth_l[l], h->d_vmap_l[l], h->d_nmap_l[l], h->d_pv_l[l], h->d_pn_l[l]};
        for (void* p : lv)
            if (p) cudaFree(p);
    }
    if (h->h_raw) cudaFreeHost(h->h_raw);
    if (h->h_state) cudaFreeHost(h->h_state);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {h->ev_pose, h->ev_fork, h->ev_join, h->ev_copied, h->ev_raw_free[0], h->ev_raw_free[1]})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : {h->aux_stream, h->pose_stream, h->copy_stream})
        if (st) cudaStreamDestroy(st);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

kf_status upload_spatial(kf_handle* h)
{
    // SystemUtility::CreateSpatialKernel + GaussianDistanceWeight
    // (system_utility.cpp:94-113): exp(-(dx^2 + dy^2) / (2 sigma_d^2)), row = dy
    const int r = h->cfg.bilateral_radius, kl = 2 * r + 1;
    std::vector<float> w((size_t)kl * kl);
    for (int y = -r; y <= r; ++y)
        for (int x = -r; x <= r; ++x) {
            const float e = -((float)(x * x) + (float)(y * y)) / (2 * h->cfg.sigma_d * h->cfg.sigma_d);
            w[(y + r) * kl + (x + r)] = (float)std::exp((double)e);
        }
    KF_CUDA(h, cudaMemcpy(h->d_spatial, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice));
    return KF_OK;
}

}  // namespace

extern "C" {

void kf_config_default(kf_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->height = 480;
    c->width = 640;
    c->min_depth = 300.f;
    c->max_depth = 2000.f;
    c->dims[0] = 360;
    c->dims[1] = 360;
    c->dims[2] = 300;
    c->grid_start[0] = -200;
    c->grid_start[1] = -200;
    c->grid_start[2] = -120;
    c->voxel_size = 10.f;
    c->truncated_distance = 300.f;
    c->sdf_minimum = -30.f;
    c->sdf_maximum = 300.f;
    c->icp_levels = 1;
    c->icp_iterations[0] = 10;
    c->icp_distance = 20.f;
    c->icp_angle_deg = 30.f;
    c->icp_fail_mode = KF_ICP_FAIL_REFERENCE;
    c->icp_reduction = KF_REDUCE_REFERENCE_ORDER;
    c->solve_mode = KF_SOLVE_REFERENCE;
    c->tsdf_storage = KF_TSDF_F32;
    c->bilateral = 0;
    c->bilateral_radius = 3;
    c->sigma_d = 4.5f;
    c->sigma_r = 30.f;
    c->use_graphs = 1;
}

const char* kf_status_string(kf_status s)
{
    switch (s) {
    case KF_OK: return "ok";
    case KF_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KF_ERR_CUDA: return "CUDA error";
    case KF_ERR_OUT_OF_MEMORY: return "out of device memory";
    case KF_ERR_STATE: return "invalid state";
    case KF_ERR_IO: return "I/O error";
    case KF_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

kf_status kf_create(const kf_config* cfg, kf_handle** out)
{
    if (!cfg || !out) return KF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::string why;
    if (!validate(cfg, why)) return KF_ERR_INVALID_ARGUMENT;
    kf_handle* h = new kf_handle;
    h->cfg = *cfg;
    cudaGetDevice(&h->device);
    h->grid = Grid{cfg->dims[0], cfg->dims[1], cfg->dims[2], cfg->grid_start[0], cfg->grid_start[1],
                   cfg->grid_start[2], cfg->voxel_size, cfg->truncated_distance, cfg->sdf_minimum, cfg->sdf_maximum,
                   div_magic((uint32_t)cfg->dims[0]), div_magic((uint32_t)cfg->dims[1])};
    h->cam.H = cfg->height;
    h->cam.W = cfg->width;
    // the reference's intrinsics (kinfu_pipeline.cpp:14-24)
    set_camera(h, 524.639f, 523.503f, 316.625f, 256.2318f);
    h->icp = IcpParams{cfg->icp_distance, cfg->icp_angle_deg, cfg->icp_fail_mode,
                       cfg->solve_mode == KF_SOLVE_PRECISE ? 1 : 0,
                       cfg->icp_reduction == KF_REDUCE_REFERENCE_ORDER ? 1 : 0};
    h->nvox = (size_t)cfg->dims[0] * cfg->dims[1] * cfg->dims[2];
    h->skip_from = float_guard_start(cfg->dims);
    kf_status s = KF_OK;
    if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) s = KF_ERR_CUDA;
    h->stream = h->own_stream;
    if (s == KF_OK) s = allocate(h);
    if (s == KF_OK) {
        icp_prepare(h->cam.H, h->cam.W);
        raycast_blocks();
        integrate_blocks();
    }
    if (s == KF_OK && cfg->bilateral) s = upload_spatial(h);
    if (s == KF_OK) s = reset_state(h);
    if (s != KF_OK) {
        free_all(h);
        delete h;
        return s;
    }
    *out = h;
    return KF_OK;
}

kf_status kf_destroy(kf_handle* h)
{
    if (!h) return KF_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return KF_OK;
}

const char* kf_last_error(const kf_handle* h) { return h ? h->err.c_str() : "null handle"; }

kf_status kf_get_config(const kf_handle* h, kf_config* cfg)
{
    if (!h || !cfg) return KF_ERR_INVALID_ARGUMENT;
    *cfg = h->cfg;
    return KF_OK;
}

kf_status kf_set_intrinsics(kf_handle* h, float fx, float fy, float cx, float cy)
{
    KF_HANDLE(h);
    if (!(fx > 0) || !(fy > 0) || !std::isfinite(cx) || !std::isfinite(cy))
        return fail(h, KF_ERR_INVALID_ARGUMENT, "intrinsics must be finite with positive focal lengths");
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    set_camera(h, fx, fy, cx, cy);
    destroy_graphs(h);  // the intrinsics are kernel arguments baked into the graphs
    return KF_OK;
}

kf_status kf_set_intrinsics_ex(kf_handle* h, float fx, float fy, float cx, float cy, int one_based)
{
    return one_based ? kf_set_intrinsics(h, fx, fy, cx, cy) : kf_set_intrinsics(h, fx, fy, cx + 1.f, cy + 1.f);
}

kf_status kf_get_intrinsics(const kf_handle* h, float K[9])
{
    if (!h || !K) return KF_ERR_INVALID_ARGUMENT;
    std::memcpy(K, h->cam.K, sizeof(float) * 9);
    return KF_OK;
}

kf_status kf_set_pose(kf_handle* h, const float T[16])
{
    KF_HANDLE(h);
    if (!T) return fail(h, KF_ERR_INVALID_ARGUMENT, "null pose");
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(T[k])) return fail(h, KF_ERR_INVALID_ARGUMENT, "pose has a non-finite entry");
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    std::memcpy(h->h_state->T, T, sizeof(float) * 16);
    for (int k = 0; k < 16; ++k) h->h_state->Td[k] = (double)T[k];
    KF_CUDA(h, cudaMemcpyAsync(field_ptr<float>(h->d_state, offsetof(State, T)), h->h_state->T, sizeof(float) * 16,
                               cudaMemcpyHostToDevice, h->stream));
    KF_CUDA(h, cudaMemcpyAsync(field_ptr<double>(h->d_state, offsetof(State, Td)), h->h_state->Td,
                               sizeof(double) * 16, cudaMemcpyHostToDevice, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_get_pose(kf_handle* h, float T[16])
{
    KF_HANDLE(h);
    if (!T) return fail(h, KF_ERR_INVALID_ARGUMENT, "null pose");
    // T and the error flag are adjacent in State: one small copy reads both
    constexpr size_t bytes = offsetof(State, error) + sizeof(int);
    if (h->pose_call + 1 == h->calls) {
        // right after a frame call: the pose is final at ev_pose; integration and the
        // ray cast go on in the stream (no kernel after the ICP writes T or the flag)
        KF_CUDA(h, cudaStreamWaitEvent(h->aux_stream, h->ev_pose, 0));
        KF_CUDA(h, cudaMemcpyAsync(h->h_state, h->d_state, bytes, cudaMemcpyDeviceToHost, h->aux_stream));
        KF_CUDA(h, cudaStreamSynchronize(h->aux_stream));
    } else {
        KF_CUDA(h, cudaMemcpyAsync(h->h_state, h->d_state, bytes, cudaMemcpyDeviceToHost, h->stream));
        KF_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    std::memcpy(T, h->h_state->T, sizeof(float) * 16);
    if (h->h_state->error) {
        const int zero = 0;
        cudaMemcpy(field_ptr<int>(h->d_state, offsetof(State, error)), &zero, sizeof(int), cudaMemcpyHostToDevice);
        return fail(h, KF_ERR_CUDA, "a kernel's bounded wait for a bulk copy gave up; the pose was not updated");
    }
    return KF_OK;
}

kf_status kf_reset(kf_handle* h)
{
    KF_HANDLE(h);
    KF_TRY(enqueue_clear(h));
    launch_state_reset(h->d_state, h->stream);
    KF_CHECK_LAUNCH(h);
    return KF_OK;
}

kf_status kf_synchronize(kf_handle* h)
{
    KF_HANDLE(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->frame_timed) {
        h->frame_timed = false;
        for (int k = 0; k < 4; ++k) cudaEventElapsedTime(&h->stage_ms[k], h->ev[k], h->ev[k + 1]);
        cudaEventElapsedTime(&h->stage_ms[4], h->ev[0], h->ev[4]);
    }
    return KF_OK;
}

kf_status kf_set_stream(kf_handle* h, void* stream)
{
    KF_HANDLE(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    return KF_OK;
}

kf_status kf_initial_processing(kf_handle* h, const uint16_t* depth)
{
    KF_HANDLE(h);
    if (!depth) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    KF_TRY(upload_raw(h, depth));
    KF_TRY(run_captured(h, h->g_initial, false, h->d_raw));
    raw_used(h, 0);
    h->pose_call = h->calls;
    return KF_OK;
}

kf_status kf_incoming_frame(kf_handle* h, const uint16_t* depth)
{
    KF_HANDLE(h);
    if (!depth) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    if (is_pinned(depth)) {
        int buf = 0;
        KF_TRY(upload_raw_async(h, depth, cudaMemcpyHostToDevice, buf));
        KF_TRY(run_captured(h, buf ? h->g_incoming_alt : h->g_incoming, true, buf ? h->d_raw_alt : h->d_raw));
        raw_used(h, buf);
    } else {
        KF_TRY(upload_raw(h, depth));
        KF_TRY(run_captured(h, h->g_incoming, true, h->d_raw));
        raw_used(h, 0);
    }
    h->frame_timed = h->timing;
    h->pose_call = h->calls;
    return KF_OK;
}

kf_status kf_process_frame(kf_handle* h, const uint16_t* depth, int is_first)
{
    return is_first ? kf_initial_processing(h, depth) : kf_incoming_frame(h, depth);
}

kf_status kf_initial_processing_device(kf_handle* h, const uint16_t* depth_dev)
{
    KF_HANDLE(h);
    if (!depth_dev) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    KF_CUDA(h, cudaMemcpyAsync(h->d_raw, depth_dev, sizeof(uint16_t) * h->cam.H * h->cam.W, cudaMemcpyDeviceToDevice,
                               h->stream));
    KF_TRY(run_captured(h, h->g_initial, false, h->d_raw));
    raw_used(h, 0);
    h->pose_call = h->calls;
    return KF_OK;
}

// The incoming-frame graph for device-resident input: captured like g_incoming, with
// the vertex kernel's node and arguments kept so that each frame points its raw input
// at the caller's buffer (the graph then reads it in stream order, with no copy).
kf_status capture_device_graph(kf_handle* h)
{
    KF_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enq_incoming(h, h->d_raw);
    cudaError_t le = cudaGetLastError();
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(h, KF_ERR_CUDA, std::string("graph capture failed: ") + cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    size_t n = 0;
    cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    cudaGraphGetNodes(graph, nodes.data(), &n);
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams p{};
        if (cudaGraphKernelNodeGetParams(nd, &p) == cudaSuccess && p.func == vertex_raw_kernel_func()) {
            h->dev_node = nd;
            h->dev_params = p;
            for (int i = 0; i < kVertexKernelArgs; ++i) h->dev_args[i] = p.kernelParams[i];
            break;
        }
    }
    cudaError_t ie = h->dev_node ? cudaGraphInstantiate(&h->g_incoming_dev, graph, 0) : cudaErrorInvalidValue;
    if (ie != cudaSuccess) {
        cudaGraphDestroy(graph);
        h->dev_node = nullptr;
        h->g_incoming_dev = nullptr;
        return fail(h, KF_ERR_CUDA, std::string("device-input graph: ") + cudaGetErrorString(ie));
    }
    h->g_dev_graph = graph;  // the node handle stays valid while the graph lives
    return KF_OK;
}

kf_status kf_incoming_frame_device(kf_handle* h, const uint16_t* depth_dev)
{
    KF_HANDLE(h);
    if (!depth_dev) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    if (h->cfg.use_graphs) {
        if (!h->g_incoming_dev) KF_TRY(capture_device_graph(h));
        h->dev_raw = depth_dev;
        h->dev_args[0] = &h->dev_raw;
        cudaKernelNodeParams p = h->dev_params;
        p.kernelParams = h->dev_args;
        KF_CUDA(h, cudaGraphExecKernelNodeSetParams(h->g_incoming_dev, h->dev_node, &p));
        KF_CUDA(h, cudaGraphLaunch(h->g_incoming_dev, h->stream));
    } else {
        // in stream order: the caller may have produced the frame on this stream
        KF_CUDA(h, cudaMemcpyAsync(h->d_raw, depth_dev, sizeof(uint16_t) * h->cam.H * h->cam.W,
                                   cudaMemcpyDeviceToDevice, h->stream));
        KF_TRY(run_captured(h, h->g_incoming, true, h->d_raw));
        raw_used(h, 0);
    }
    h->frame_timed = h->timing;
    h->pose_call = h->calls;
    return KF_OK;
}

kf_status kf_load_depth_dat(const char* dir, int frame_index, int height, int width, uint16_t* depth)
{
    if (!dir || !depth || height <= 0 || width <= 0) return KF_ERR_INVALID_ARGUMENT;
    char path[4096];
    std::snprintf(path, sizeof(path), "%s/dep%04d.dat", dir, frame_index);
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return KF_ERR_IO;
    const size_t n = (size_t)height * width;
    const size_t got = std::fread(depth, sizeof(uint16_t), n, fp);
    std::fclose(fp);
    return got == n ? KF_OK : KF_ERR_IO;
}

kf_status kf_get_predicted(kf_handle* h, float* x, float* y, float* z, float* nx, float* ny, float* nz)
{
    KF_HANDLE(h);
    const size_t HW = (size_t)h->cam.H * h->cam.W;
    std::vector<float4> pv(HW), pn(HW);
    KF_CUDA(h, cudaMemcpyAsync(pv.data(), h->d_pv, sizeof(float4) * HW, cudaMemcpyDeviceToHost, h->stream));
    KF_CUDA(h, cudaMemcpyAsync(pn.data(), h->d_pn, sizeof(float4) * HW, cudaMemcpyDeviceToHost, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < HW; ++i) {
        if (x) x[i] = pv[i].x;
        if (y) y[i] = pv[i].y;
        if (z) z[i] = pv[i].z;
        if (nx) nx[i] = pn[i].x;
        if (ny) ny[i] = pn[i].y;
        if (nz) nz[i] = pn[i].z;
    }
    return KF_OK;
}

kf_status kf_set_predicted(kf_handle* h, const float* x, const float* y, const float* z, const float* nx,
                           const float* ny, const float* nz)
{
    KF_HANDLE(h);
    if (!x || !y || !z || !nx || !ny || !nz) return fail(h, KF_ERR_INVALID_ARGUMENT, "null plane");
    const size_t HW = (size_t)h->cam.H * h->cam.W;
    std::vector<float4> pv(HW), pn(HW);
    for (size_t i = 0; i < HW; ++i) {
        pv[i] = make_float4(x[i], y[i], z[i], 0.f);
        pn[i] = make_float4(nx[i], ny[i], nz[i], 0.f);
    }
    KF_CUDA(h, cudaMemcpyAsync(h->d_pv, pv.data(), sizeof(float4) * HW, cudaMemcpyHostToDevice, h->stream));
    KF_CUDA(h, cudaMemcpyAsync(h->d_pn, pn.data(), sizeof(float4) * HW, cudaMemcpyHostToDevice, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_get_volume(kf_handle* h, float* tsdf, float* weight)
{
    KF_HANDLE(h);
    float *dt = nullptr, *dw = nullptr;
    KF_CUDA(h, cudaMalloc((void**)&dt, sizeof(float) * h->nvox));
    cudaError_t e = cudaMalloc((void**)&dw, sizeof(float) * h->nvox);
    if (e != cudaSuccess) {
        cudaFree(dt);
        return fail(h, KF_ERR_OUT_OF_MEMORY, "volume readback buffer");
    }
    if (h->d_vol16) {
        launch_half2_to_zfast(h->d_vol16, dt, dw, h->grid, h->stream);
    } else {
        launch_to_zfast_f32(h->d_tsdf, dt, h->grid, h->stream);
        launch_to_zfast_f32(h->d_weight, dw, h->grid, h->stream);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess && tsdf)
        e = cudaMemcpyAsync(tsdf, dt, sizeof(float) * h->nvox, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && weight)
        e = cudaMemcpyAsync(weight, dw, sizeof(float) * h->nvox, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dt);
    cudaFree(dw);
    if (e != cudaSuccess) return fail(h, KF_ERR_CUDA, std::string("kf_get_volume: ") + cudaGetErrorString(e));
    return KF_OK;
}

kf_status kf_set_volume(kf_handle* h, const float* tsdf, const float* weight)
{
    KF_HANDLE(h);
    if (!tsdf || !weight) return fail(h, KF_ERR_INVALID_ARGUMENT, "null volume");
    float *dt = nullptr, *dw = nullptr;
    KF_CUDA(h, cudaMalloc((void**)&dt, sizeof(float) * h->nvox));
    cudaError_t e = cudaMalloc((void**)&dw, sizeof(float) * h->nvox);
    if (e != cudaSuccess) {
        cudaFree(dt);
        return fail(h, KF_ERR_OUT_OF_MEMORY, "volume upload buffer");
    }
    e = cudaMemcpyAsync(dt, tsdf, sizeof(float) * h->nvox, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw, weight, sizeof(float) * h->nvox, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        if (h->d_vol16) {
            launch_zfast_to_half2(dt, dw, h->d_vol16, h->grid, h->stream);
        } else {
            launch_from_zfast_f32(dt, h->d_tsdf, h->grid, h->stream);
            launch_from_zfast_f32(dw, h->d_weight, h->grid, h->stream);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dt);
    cudaFree(dw);
    if (e != cudaSuccess) return fail(h, KF_ERR_CUDA, std::string("kf_set_volume: ") + cudaGetErrorString(e));
    return KF_OK;
}

kf_status kf_export_ply(kf_handle* h, const char* path, const uint8_t* colour_bgr, int* n_points)
{
    KF_HANDLE(h);
    if (!path) return fail(h, KF_ERR_INVALID_ARGUMENT, "null path");
    const int n = h->cam.H * h->cam.W;
    float4* d_cloud = nullptr;
    unsigned* d_count = nullptr;
    KF_CUDA(h, cudaMalloc((void**)&d_cloud, sizeof(float4) * 2 * (size_t)n + sizeof(unsigned)));
    d_count = reinterpret_cast<unsigned*>(d_cloud + 2 * (size_t)n);
    cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(unsigned), h->stream);
    if (e == cudaSuccess) {
        launch_compact_cloud(h->d_pv, h->d_pn, n, d_cloud, d_count, h->stream);
        e = cudaGetLastError();
    }
    unsigned count = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&count, d_count, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    std::vector<float4> cloud(2 * (size_t)count);
    if (e == cudaSuccess && count)
        e = cudaMemcpy(cloud.data(), d_cloud, sizeof(float4) * cloud.size(), cudaMemcpyDeviceToHost);
    cudaFree(d_cloud);
    if (e != cudaSuccess) return fail(h, KF_ERR_CUDA, std::string("kf_export_ply: ") + cudaGetErrorString(e));
    // pixel order, as the viewer fills its cloud
    std::vector<unsigned> order(count);
    for (unsigned k = 0; k < count; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](unsigned a, unsigned b) {
        return __builtin_bit_cast(int, cloud[2 * a].w) < __builtin_bit_cast(int, cloud[2 * b].w);
    });
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(h, KF_ERR_IO, std::string("cannot open ") + path);
    std::fprintf(f,
                 "ply\nformat binary_little_endian 1.0\ncomment kinfu_gb300 predicted surface, mm, world frame\n"
                 "element vertex %u\nproperty float x\nproperty float y\nproperty float z\nproperty float nx\n"
                 "property float ny\nproperty float nz\nproperty uchar red\nproperty uchar green\n"
                 "property uchar blue\nend_header\n",
                 count);
    bool ok = true;
    for (unsigned k = 0; k < count && ok; ++k) {
        const float4 p = cloud[2 * order[k]], q = cloud[2 * order[k] + 1];
        const int pix = __builtin_bit_cast(int, p.w);
        unsigned char rgb[3];
        if (colour_bgr) {
            rgb[0] = colour_bgr[3 * (size_t)pix + 2];
            rgb[1] = colour_bgr[3 * (size_t)pix + 1];
            rgb[2] = colour_bgr[3 * (size_t)pix];
        } else {
            const float c[3] = {q.x, q.y, q.z};
            for (int j = 0; j < 3; ++j) {
                const float v = std::isfinite(c[j]) ? 127.5f * (c[j] + 1.f) : 0.f;
                rgb[j] = (unsigned char)(v < 0.f ? 0.f : (v > 255.f ? 255.f : v));
            }
        }
        const float rec[6] = {p.x, p.y, p.z, q.x, q.y, q.z};
        // the record is little-endian floats then bytes; both build hosts are little-endian
        ok = std::fwrite(rec, sizeof(float), 6, f) == 6 && std::fwrite(rgb, 1, 3, f) == 3;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(h, KF_ERR_IO, std::string("short write to ") + path);
    if (n_points) *n_points = (int)count;
    return KF_OK;
}

namespace {

// checkpoint file: this header, then the volume in the device layout (FP32: value plane
// then weight plane; FP16: the half2 plane), then the predicted points and normals
struct CheckpointHeader {
    char magic[8];
    uint32_t version;
    int32_t height, width, dims[3], start[3], storage;
    float voxel_size, truncated_distance, sdf_minimum, sdf_maximum;
    float K[9];
    float T[16];
    double Td[16];
    uint64_t volume_bytes, prediction_bytes;
};
constexpr char kCheckpointMagic[8] = {'K', 'F', 'G', 'B', '3', '0', '0', '\0'};

void fill_header(const kf_handle* h, CheckpointHeader& c)
{
    std::memset(&c, 0, sizeof(c));
    std::memcpy(c.magic, kCheckpointMagic, sizeof(c.magic));
    c.version = 1;
    c.height = h->cfg.height;
    c.width = h->cfg.width;
    for (int k = 0; k < 3; ++k) {
        c.dims[k] = h->cfg.dims[k];
        c.start[k] = h->cfg.grid_start[k];
    }
    c.storage = h->cfg.tsdf_storage;
    c.voxel_size = h->cfg.voxel_size;
    c.truncated_distance = h->cfg.truncated_distance;
    c.sdf_minimum = h->cfg.sdf_minimum;
    c.sdf_maximum = h->cfg.sdf_maximum;
    for (int k = 0; k < 9; ++k) c.K[k] = h->cam.K[k];
    c.volume_bytes = h->d_vol16 ? sizeof(__half2) * h->nvox : 2 * sizeof(float) * h->nvox;
    c.prediction_bytes = 2 * sizeof(float4) * (size_t)h->cam.H * h->cam.W;
}

// streams count bytes between a device buffer and a file through a pinned staging buffer
bool stream_file(FILE* f, void* dev, size_t count, bool to_file, cudaStream_t s)
{
    constexpr size_t kChunk = 64u << 20;
    void* stage = nullptr;
    if (cudaMallocHost(&stage, kChunk) != cudaSuccess) return false;
    bool ok = true;
    for (size_t off = 0; off < count && ok; off += kChunk) {
        const size_t n = count - off < kChunk ? count - off : kChunk;
        char* d = static_cast<char*>(dev) + off;
        if (to_file) {
            ok = cudaMemcpyAsync(stage, d, n, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                 cudaStreamSynchronize(s) == cudaSuccess && std::fwrite(stage, 1, n, f) == n;
        } else {
            ok = std::fread(stage, 1, n, f) == n &&
                 cudaMemcpyAsync(d, stage, n, cudaMemcpyHostToDevice, s) == cudaSuccess &&
                 cudaStreamSynchronize(s) == cudaSuccess;
        }
    }
    cudaFreeHost(stage);
    return ok;
}

}  // namespace

kf_status kf_save_checkpoint(kf_handle* h, const char* path)
{
    KF_HANDLE(h);
    if (!path) return fail(h, KF_ERR_INVALID_ARGUMENT, "null path");
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    KF_CUDA(h, cudaMemcpy(h->h_state, h->d_state, sizeof(State), cudaMemcpyDeviceToHost));
    CheckpointHeader c;
    fill_header(h, c);
    std::memcpy(c.T, h->h_state->T, sizeof(c.T));
    std::memcpy(c.Td, h->h_state->Td, sizeof(c.Td));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(h, KF_ERR_IO, std::string("cannot open ") + path);
    bool ok = std::fwrite(&c, sizeof(c), 1, f) == 1;
    const size_t plane = sizeof(float) * h->nvox, img = sizeof(float4) * (size_t)h->cam.H * h->cam.W;
    if (h->d_vol16) {
        ok = ok && stream_file(f, h->d_vol16, sizeof(__half2) * h->nvox, true, h->stream);
    } else {
        ok = ok && stream_file(f, h->d_tsdf, plane, true, h->stream);
        ok = ok && stream_file(f, h->d_weight, plane, true, h->stream);
    }
    ok = ok && stream_file(f, h->d_pv, img, true, h->stream) && stream_file(f, h->d_pn, img, true, h->stream);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(h, KF_ERR_IO, std::string("writing checkpoint ") + path + " failed");
    return KF_OK;
}

kf_status kf_load_checkpoint(kf_handle* h, const char* path)
{
    KF_HANDLE(h);
    if (!path) return fail(h, KF_ERR_INVALID_ARGUMENT, "null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(h, KF_ERR_IO, std::string("cannot open ") + path);
    CheckpointHeader c, want;
    fill_header(h, want);
    if (std::fread(&c, sizeof(c), 1, f) != 1 || std::memcmp(c.magic, kCheckpointMagic, sizeof(c.magic)) != 0 ||
        c.version != 1) {
        std::fclose(f);
        return fail(h, KF_ERR_IO, std::string(path) + " is not a kinfu_gb300 checkpoint");
    }
    const bool same = c.height == want.height && c.width == want.width && c.storage == want.storage &&
                      std::memcmp(c.dims, want.dims, sizeof(c.dims)) == 0 &&
                      std::memcmp(c.start, want.start, sizeof(c.start)) == 0 && c.voxel_size == want.voxel_size &&
                      c.truncated_distance == want.truncated_distance && c.sdf_minimum == want.sdf_minimum &&
                      c.sdf_maximum == want.sdf_maximum && c.volume_bytes == want.volume_bytes &&
                      c.prediction_bytes == want.prediction_bytes;
    if (!same) {
        std::fclose(f);
        return fail(h, KF_ERR_INVALID_ARGUMENT, "checkpoint was saved with another image size, grid or storage");
    }
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(c.T[k]) || !std::isfinite(c.Td[k])) {
            std::fclose(f);
            return fail(h, KF_ERR_IO, "checkpoint pose has a non-finite entry");
        }
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    const size_t plane = sizeof(float) * h->nvox, img = sizeof(float4) * (size_t)h->cam.H * h->cam.W;
    bool ok;
    if (h->d_vol16) {
        ok = stream_file(f, h->d_vol16, sizeof(__half2) * h->nvox, false, h->stream);
    } else {
        ok = stream_file(f, h->d_tsdf, plane, false, h->stream) && stream_file(f, h->d_weight, plane, false, h->stream);
    }
    ok = ok && stream_file(f, h->d_pv, img, false, h->stream) && stream_file(f, h->d_pn, img, false, h->stream);
    std::fclose(f);
    if (!ok) return fail(h, KF_ERR_IO, std::string("reading checkpoint ") + path + " failed");
    kf_status s = kf_set_intrinsics(h, c.K[0], c.K[4], c.K[2], c.K[5]);
    if (s != KF_OK) return s;
    std::memcpy(h->h_state->T, c.T, sizeof(c.T));
    std::memcpy(h->h_state->Td, c.Td, sizeof(c.Td));
    KF_CUDA(h, cudaMemcpy(field_ptr<float>(h->d_state, offsetof(State, T)), c.T, sizeof(c.T), cudaMemcpyHostToDevice));
    KF_CUDA(h, cudaMemcpy(field_ptr<double>(h->d_state, offsetof(State, Td)), c.Td, sizeof(c.Td),
                          cudaMemcpyHostToDevice));
    return KF_OK;
}

kf_status kf_get_depth(kf_handle* h, float* depth)
{
    KF_HANDLE(h);
    if (!depth) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    KF_CUDA(h, cudaMemcpyAsync(depth, h->d_depth, sizeof(float) * h->cam.H * h->cam.W, cudaMemcpyDeviceToHost,
                               h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_get_icp_stats(kf_handle* h, int32_t* ncorr, int32_t* chol_ok, float* poses, int n)
{
    KF_HANDLE(h);
    if (n < 0) return fail(h, KF_ERR_INVALID_ARGUMENT, "negative count");
    KF_TRY(read_state(h));
    const int m = n < kMaxIcpIters ? n : kMaxIcpIters;
    for (int k = 0; k < m; ++k) {
        if (ncorr) ncorr[k] = h->h_state->ncorr[k];
        if (chol_ok) chol_ok[k] = h->h_state->chol_ok[k];
        if (poses) std::memcpy(poses + 16 * k, h->h_state->Tlog[k], sizeof(float) * 16);
    }
    return KF_OK;
}

kf_status kf_set_depth_f32(kf_handle* h, const float* depth)
{
    KF_HANDLE(h);
    if (!depth) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    KF_CUDA(h, cudaMemcpyAsync(h->d_depth, depth, sizeof(float) * h->cam.H * h->cam.W, cudaMemcpyHostToDevice,
                               h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_set_depth_u16(kf_handle* h, const uint16_t* depth)
{
    KF_HANDLE(h);
    if (!depth) return fail(h, KF_ERR_INVALID_ARGUMENT, "null depth");
    KF_TRY(upload_raw(h, depth));
    enq_ingest(h, h->d_raw, false, false);
    raw_used(h, 0);
    KF_CHECK_LAUNCH(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_calculate_vertices_and_normals(kf_handle* h, float* vx, float* vy, float* nx, float* ny, float* nz,
                                            uint8_t* mask)
{
    KF_HANDLE(h);
    enq_ingest(h, nullptr, false, true);
    KF_CHECK_LAUNCH(h);
    if (!vx && !vy && !nx && !ny && !nz && !mask) {
        KF_CUDA(h, cudaStreamSynchronize(h->stream));
        return KF_OK;
    }
    const size_t HW = (size_t)h->cam.H * h->cam.W;
    std::vector<float4> v(HW), n(HW);
    KF_CUDA(h, cudaMemcpyAsync(v.data(), h->d_vmap, sizeof(float4) * HW, cudaMemcpyDeviceToHost, h->stream));
    KF_CUDA(h, cudaMemcpyAsync(n.data(), h->d_nmap, sizeof(float4) * HW, cudaMemcpyDeviceToHost, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < HW; ++i) {
        if (vx) vx[i] = v[i].x;
        if (vy) vy[i] = v[i].y;
        if (nx) nx[i] = n[i].x;
        if (ny) ny[i] = n[i].y;
        if (nz) nz[i] = n[i].z;
        if (mask) mask[i] = v[i].w != 0.f ? 1 : 0;
    }
    return KF_OK;
}

kf_status kf_bilateral_filtering(kf_handle* h)
{
    KF_HANDLE(h);
    if (!h->cfg.bilateral) {
        // the spatial kernel is uploaded on first use for handles created without it
        h->cfg.bilateral = 1;
        kf_status s = upload_spatial(h);
        h->cfg.bilateral = 0;
        if (s != KF_OK) return s;
    }
    enq_bilateral(h);
    KF_CHECK_LAUNCH(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_estimate_sensor_pose(kf_handle* h)
{
    KF_HANDLE(h);
    // re-derive the frame-start ICP state from the current pose; the vertex map is
    // left as the last kf_calculate_vertices_and_normals produced it
    launch_vertex(nullptr, h->d_depth, h->d_vmap, h->d_nmap, h->cam, h->cfg.min_depth, h->cfg.max_depth,
                  h->d_state, true, false, h->stream);
    enq_icp(h);
    KF_CHECK_LAUNCH(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_projective_tsdf(kf_handle* h, int first_tsdf_construct)
{
    KF_HANDLE(h);
    enq_integrate(h, first_tsdf_construct != 0);
    KF_CHECK_LAUNCH(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_ray_casting(kf_handle* h, int32_t* hit)
{
    KF_HANDLE(h);
    enq_raycast(h, h->d_hit);
    KF_CHECK_LAUNCH(h);
    if (hit)
        KF_CUDA(h, cudaMemcpyAsync(hit, h->d_hit, sizeof(int32_t) * h->cam.H * h->cam.W, cudaMemcpyDeviceToHost,
                                   h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_icp_associate(kf_handle* h, const float F[16], const float T[16], int32_t* pair, float* sums27,
                           int32_t* ncorr)
{
    KF_HANDLE(h);
    if (!F || !T) return fail(h, KF_ERR_INVALID_ARGUMENT, "null transform");
    float mats[32];
    std::memcpy(mats, F, sizeof(float) * 16);
    std::memcpy(mats + 16, T, sizeof(float) * 16);
    KF_CUDA(h, cudaMemcpyAsync(h->d_mats, mats, sizeof(mats), cudaMemcpyHostToDevice, h->stream));
    launch_icp_associate(h->d_vmap, h->d_nmap, h->d_pv, h->d_pn, h->cam, h->icp, h->d_mats, h->d_mats + 16,
                         h->d_state, h->d_partials, h->d_groups, h->d_fixacc, h->d_mats + 32,
                         pair ? h->d_pair : nullptr, h->stream);
    KF_CHECK_LAUNCH(h);
    float sums[kIcpVals];
    KF_CUDA(h, cudaMemcpyAsync(sums, h->d_mats + 32, sizeof(sums), cudaMemcpyDeviceToHost, h->stream));
    if (pair)
        KF_CUDA(h, cudaMemcpyAsync(pair, h->d_pair, sizeof(int32_t) * h->cam.H * h->cam.W, cudaMemcpyDeviceToHost,
                                   h->stream));
    int err = 0;
    KF_CUDA(h, cudaMemcpyAsync(&err, field_ptr<int>(h->d_state, offsetof(State, error)), sizeof(int),
                               cudaMemcpyDeviceToHost, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    if (err) {
        const int zero = 0;
        KF_CUDA(h, cudaMemcpy(field_ptr<int>(h->d_state, offsetof(State, error)), &zero, sizeof(int),
                              cudaMemcpyHostToDevice));
        return fail(h, KF_ERR_CUDA, "the reduction's bounded wait for a bulk copy gave up; no sums were produced");
    }
    if (sums27) std::memcpy(sums27, sums, sizeof(float) * 27);
    if (ncorr) *ncorr = (int32_t)sums[kIcpVals - 1];
    return KF_OK;
}

kf_status kf_get_flip_threshold(kf_handle* h, float* c_flip)
{
    KF_HANDLE(h);
    if (!c_flip) return fail(h, KF_ERR_INVALID_ARGUMENT, "null output");
    KF_TRY(read_state(h));
    *c_flip = h->h_state->c_flip;
    return KF_OK;
}

kf_status kf_enable_stage_timing(kf_handle* h, int enable)
{
    KF_HANDLE(h);
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    if ((enable != 0) != h->timing) {
        h->timing = enable != 0;
        destroy_graphs(h);
    }
    return KF_OK;
}

kf_status kf_get_stage_times(kf_handle* h, float ms[5])
{
    KF_HANDLE(h);
    if (!ms) return fail(h, KF_ERR_INVALID_ARGUMENT, "null output");
    KF_TRY(kf_synchronize(h));
    std::memcpy(ms, h->stage_ms, sizeof(float) * 5);
    return KF_OK;
}

kf_status kf_set_wait_limit(kf_handle* h, long long polls)
{
    KF_HANDLE(h);
    const long long v = polls < 0 ? kf::kDefaultWaitLimit : polls;
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    h->h_state->wait_limit = v;
    KF_CUDA(h, cudaMemcpyAsync(field_ptr<long long>(h->d_state, offsetof(State, wait_limit)), &h->h_state->wait_limit,
                               sizeof(long long), cudaMemcpyHostToDevice, h->stream));
    KF_CUDA(h, cudaStreamSynchronize(h->stream));
    return KF_OK;
}

kf_status kf_kernels_per_frame(kf_handle* h, int* n)
{
    if (!h || !n) return KF_ERR_INVALID_ARGUMENT;
    // vertex, [bilateral], ICP iterations (in the reference summation order a 64-pixel
    // group pass and a one-warp reduce-and-solve pass; the precision form and the tree
    // reduction one pass each), integration prep, box marks, mark list, integration, ray cast
    const int per_iteration =
        (h->cfg.icp_reduction == KF_REDUCE_REFERENCE_ORDER && h->cfg.solve_mode != KF_SOLVE_PRECISE) ? 2 : 1;
    int iterations = 0;
    for (int l = 0; l < h->cfg.icp_levels; ++l) iterations += h->cfg.icp_iterations[l];
    *n = 1 + (h->cfg.bilateral ? 1 : 0) + 3 * (h->cfg.icp_levels - 1) + per_iteration * iterations + 5;
    return KF_OK;
}

}  // extern "C"
