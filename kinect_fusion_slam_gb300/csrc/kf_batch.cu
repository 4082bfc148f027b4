// The batching form: many independent scenes, one launch per stage for all of them and
// the whole frame as one CUDA graph (include/kinfu_gb300.h, kf_batch_*).
//
// A batch owns one ordinary kf_handle per scene and a device table of SceneDev entries
// pointing at those handles' buffers.  The batched kernels (kf_depth.cu, kf_icp.cu,
// kf_tsdf.cu) run the single-scene kernels' device code for the scene their block
// belongs to, so each scene's results are the ones its handle would compute alone.
// Per frame the host writes the table's raw-depth pointers (one small copy) and
// replays the frame's graph: vertex maps, the pyramid levels, the fixed-count ICP
// iterations (group pass + one solve CTA per scene), integration and the ray cast.
#include <algorithm>
#include <cstring>
#include <vector>

#include "kinfu_gb300.h"
#include "kf_handle.h"
#include "kf_kernels.h"

using namespace kf;

struct kf_batch {
    std::vector<kf_handle*> scenes;
    int n = 0;
    int levels = 1;
    int iters[kMaxLevels] = {};
    bool f16 = false;
    cudaStream_t stream = nullptr;
    SceneDev* h_table = nullptr;  // pinned
    SceneDev* d_table = nullptr;
    unsigned* d_tiles = nullptr;  // ray-cast tile counter pair
    int max_pixels[kMaxLevels] = {}, max_groups[kMaxLevels] = {};
    int tuning[4] = {8, 0, 4, 16};  // group warps, ray shape, ray blocks per SM, z chunk
    int sms = 152;
    // which stages run over the flattened work of all scenes on a fixed grid (1) rather
    // than as a 2-D grid with a row of blocks per scene (0): integration, ICP group pass
    int persist_int = 0, persist_icp = 0;
    unsigned* d_work = nullptr;  // integration's box counter pair
    unsigned total_boxes = 0, total_groups[kMaxLevels] = {};
    cudaGraphExec_t g_initial = nullptr, g_incoming = nullptr;
};

namespace {

void destroy_graphs(kf_batch* b)
{
    if (b->g_initial) cudaGraphExecDestroy(b->g_initial);
    if (b->g_incoming) cudaGraphExecDestroy(b->g_incoming);
    b->g_initial = b->g_incoming = nullptr;
}

// the scene table from the handles' current buffers and cameras
void fill_table(kf_batch* b)
{
    int start[3] = {0, 0, 0};
    unsigned boxes = 0, groups[kMaxLevels] = {};
    for (int i = 0; i < b->n; ++i) {
        const kf_handle* h = b->scenes[i];
        SceneDev& d = b->h_table[i];
        const uint16_t* raw = d.raw;
        std::memset(&d, 0, sizeof(d));
        d.raw = raw;
        for (int l = 0; l < kMaxLevels; ++l) {
            d.cam[l] = h->lcam[l];
            d.depth[l] = h->d_depth_l[l];
            d.vmap[l] = h->d_vmap_l[l];
            d.nmap[l] = h->d_nmap_l[l];
            d.pv[l] = h->d_pv_l[l];
            d.pn[l] = h->d_pn_l[l];
        }
        d.grid = h->grid;
        d.icp = h->icp;
        d.tab = h->d_tab;
        d.tsdf = h->d_tsdf;
        d.weight = h->d_weight;
        d.vol16 = h->d_vol16;
        d.st = h->d_state;
        d.partials = h->d_partials;
        d.groups = h->d_groups;
        d.hit = h->d_hit;
        d.skip_from = h->skip_from;
        d.dmin = h->cfg.min_depth;
        d.dmax = h->cfg.max_depth;
        d.band = 3.0f * h->cfg.sigma_r;
        d.depth_eps = depth_band_eps(h->cam);
        d.lam_max = ray_norm_max(h->cam);
        for (int sh = 0; sh < 3; ++sh) {
            d.tile_start[sh] = start[sh];
            start[sh] += raycast_tiles(h->cam.H, h->cam.W, sh);
        }
        d.int_start = (int)boxes;
        boxes += (unsigned)integrate_tiles(h->grid, b->tuning[3]);
        for (int l = 0; l < kMaxLevels; ++l) {
            d.grp_start[l] = (int)groups[l];
            groups[l] += (unsigned)((h->lcam[l].H * h->lcam[l].W + 63) / 64);
        }
    }
    b->total_boxes = boxes;
    for (int l = 0; l < kMaxLevels; ++l) b->total_groups[l] = groups[l];
}

unsigned total_ray_tiles(const kf_batch* b, int shape)
{
    unsigned t = 0;
    for (const kf_handle* h : b->scenes) t += (unsigned)raycast_tiles(h->cam.H, h->cam.W, shape);
    return t;
}

int max_integrate_tiles(const kf_batch* b, int zchunk)
{
    int m = 0;
    for (const kf_handle* h : b->scenes) m = std::max(m, integrate_tiles(h->grid, zchunk));
    return m;
}

void enq_frame(kf_batch* b, bool incoming)
{
    cudaStream_t s = b->stream;
    launch_vertex_batch(b->d_table, b->n, b->max_pixels[0], 0, incoming, s);
    if (incoming) {
        for (int l = 1; l < b->levels; ++l) {
            launch_pyramid_batch(b->d_table, b->n, b->max_pixels[l], l, s);
            launch_vertex_batch(b->d_table, b->n, b->max_pixels[l], l, false, s);
        }
        for (int l = b->levels - 1; l >= 0; --l)
            for (int it = 0; it < b->iters[l]; ++it) {
                if (b->persist_icp)
                    launch_icp_iteration_batch_persistent(b->d_table, b->n, b->max_groups[l], l, b->total_groups[l],
                                                          4 * b->sms, s);
                else
                    launch_icp_iteration_batch(b->d_table, b->n, b->max_groups[l], l, b->tuning[0], s);
            }
    }
    const int zc = b->tuning[3];
    if (b->persist_int)
        launch_integrate_batch_persistent(b->d_table, b->n, b->max_pixels[0], b->total_boxes, zc, b->f16, !incoming,
                                          5 * b->sms, b->d_work, s);
    else
        launch_integrate_batch(b->d_table, b->n, b->max_pixels[0], max_integrate_tiles(b, zc), zc, b->f16, !incoming,
                               s);
    launch_raycast_batch(b->d_table, b->n, total_ray_tiles(b, b->tuning[1]), b->f16, b->tuning[1],
                         b->tuning[2] * b->sms, b->d_tiles, s);
}

kf_status run_frame(kf_batch* b, const uint16_t* const* depth, bool incoming)
{
    if (!b || !depth) return KF_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < b->n; ++i)
        if (!depth[i]) return KF_ERR_INVALID_ARGUMENT;
    // the previous frame's table copy must have left the pinned buffer
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return KF_ERR_CUDA;
    for (int i = 0; i < b->n; ++i) b->h_table[i].raw = depth[i];
    if (cudaMemcpyAsync(b->d_table, b->h_table, sizeof(SceneDev) * b->n, cudaMemcpyHostToDevice, b->stream) !=
        cudaSuccess)
        return KF_ERR_CUDA;
    cudaGraphExec_t& exec = incoming ? b->g_incoming : b->g_initial;
    if (!exec) {
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return KF_ERR_CUDA;
        enq_frame(b, incoming);
        if (cudaStreamEndCapture(b->stream, &graph) != cudaSuccess) return KF_ERR_CUDA;
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            exec = nullptr;
            return KF_ERR_CUDA;
        }
    }
    return cudaGraphLaunch(exec, b->stream) == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}

bool same_schedule(const kf_config& a, const kf_config& c)
{
    if (a.icp_levels != c.icp_levels || a.tsdf_storage != c.tsdf_storage) return false;
    for (int l = 0; l < a.icp_levels; ++l)
        if (a.icp_iterations[l] != c.icp_iterations[l]) return false;
    return true;
}

}  // namespace

extern "C" {

kf_status kf_batch_create(const kf_config* configs, int n_scenes, kf_batch** out)
{
    if (!configs || !out || n_scenes < 1 || n_scenes > 64) return KF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    for (int i = 0; i < n_scenes; ++i) {
        const kf_config& c = configs[i];
        if (!same_schedule(configs[0], c) || c.icp_reduction != KF_REDUCE_REFERENCE_ORDER ||
            c.solve_mode != KF_SOLVE_REFERENCE || c.bilateral)
            return KF_ERR_INVALID_ARGUMENT;
    }
    kf_batch* b = new kf_batch;
    b->n = n_scenes;
    b->levels = configs[0].icp_levels;
    for (int l = 0; l < b->levels; ++l) b->iters[l] = configs[0].icp_iterations[l];
    b->f16 = configs[0].tsdf_storage == KF_TSDF_F16;
    kf_status s = KF_OK;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) s = KF_ERR_CUDA;
    for (int i = 0; i < n_scenes && s == KF_OK; ++i) {
        kf_handle* h = nullptr;
        s = kf_create(&configs[i], &h);
        if (s == KF_OK) {
            b->scenes.push_back(h);
            s = kf_set_stream(h, b->stream);
        }
    }
    if (s == KF_OK && (cudaMallocHost((void**)&b->h_table, sizeof(SceneDev) * n_scenes) != cudaSuccess ||
                       cudaMalloc((void**)&b->d_table, sizeof(SceneDev) * n_scenes) != cudaSuccess ||
                       cudaMalloc((void**)&b->d_tiles, 2 * sizeof(unsigned)) != cudaSuccess ||
                       cudaMemset(b->d_tiles, 0, 2 * sizeof(unsigned)) != cudaSuccess ||
                       cudaMalloc((void**)&b->d_work, 2 * sizeof(unsigned)) != cudaSuccess ||
                       cudaMemset(b->d_work, 0, 2 * sizeof(unsigned)) != cudaSuccess))
        s = KF_ERR_OUT_OF_MEMORY;
    if (s == KF_OK) {
        std::memset(b->h_table, 0, sizeof(SceneDev) * n_scenes);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
        for (const kf_handle* h : b->scenes)
            for (int l = 0; l < b->levels; ++l) {
                const int px = h->lcam[l].H * h->lcam[l].W;
                b->max_pixels[l] = std::max(b->max_pixels[l], px);
                b->max_groups[l] = std::max(b->max_groups[l], (px + 63) / 64);
            }
        icp_prepare(1, b->max_groups[0] * 64);
        fill_table(b);
    }
    if (s != KF_OK) {
        kf_batch_destroy(b);
        return s;
    }
    *out = b;
    return KF_OK;
}

kf_status kf_batch_destroy(kf_batch* b)
{
    if (!b) return KF_ERR_INVALID_ARGUMENT;
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroy_graphs(b);
    for (kf_handle* h : b->scenes) kf_destroy(h);
    if (b->h_table) cudaFreeHost(b->h_table);
    if (b->d_table) cudaFree(b->d_table);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->d_work) cudaFree(b->d_work);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return KF_OK;
}

kf_status kf_batch_scene(kf_batch* b, int scene, kf_handle** out)
{
    if (!b || !out || scene < 0 || scene >= b->n) return KF_ERR_INVALID_ARGUMENT;
    *out = b->scenes[scene];
    return KF_OK;
}

kf_status kf_batch_initial_processing_device(kf_batch* b, const uint16_t* const* depth)
{
    if (!b) return KF_ERR_INVALID_ARGUMENT;
    // the scene handles' intrinsics may have changed (the kernels read them from the
    // table); the pinned table must not be in flight while it is rewritten
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return KF_ERR_CUDA;
    fill_table(b);
    return run_frame(b, depth, false);
}

kf_status kf_batch_incoming_frame_device(kf_batch* b, const uint16_t* const* depth)
{
    return run_frame(b, depth, true);
}

kf_status kf_batch_synchronize(kf_batch* b)
{
    if (!b) return KF_ERR_INVALID_ARGUMENT;
    return cudaStreamSynchronize(b->stream) == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}

kf_status kf_batch_kernels_per_frame(kf_batch* b, int* n)
{
    if (!b || !n) return KF_ERR_INVALID_ARGUMENT;
    int iterations = 0;
    for (int l = 0; l < b->levels; ++l) iterations += b->iters[l];
    // vertex, 2 per extra pyramid level, 2 per ICP iteration, integration prep +
    // integration, ray cast
    *n = 1 + 2 * (b->levels - 1) + 2 * iterations + 3;
    return KF_OK;
}

kf_status kf_batch_set_tuning(kf_batch* b, const int tuning[4])
{
    if (!b || !tuning) return KF_ERR_INVALID_ARGUMENT;
    const bool ok = (tuning[0] == 4 || tuning[0] == 8 || tuning[0] == 16) && tuning[1] >= 0 && tuning[1] <= 2 &&
                    tuning[2] >= 1 && tuning[2] <= 4 && (tuning[3] == 8 || tuning[3] == 16 || tuning[3] == 32);
    if (!ok) return KF_ERR_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return KF_ERR_CUDA;
    std::memcpy(b->tuning, tuning, sizeof(b->tuning));
    fill_table(b);  // the flattened box list depends on the z chunk
    if (cudaMemcpy(b->d_table, b->h_table, sizeof(SceneDev) * b->n, cudaMemcpyHostToDevice) != cudaSuccess)
        return KF_ERR_CUDA;
    destroy_graphs(b);
    return KF_OK;
}

kf_status kf_batch_set_forms(kf_batch* b, int persistent_integration, int persistent_icp)
{
    if (!b) return KF_ERR_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return KF_ERR_CUDA;
    b->persist_int = persistent_integration != 0;
    b->persist_icp = persistent_icp != 0;
    destroy_graphs(b);
    return KF_OK;
}

kf_status kf_batch_autotune(kf_batch* b, int tuning[4])
{
    if (!b) return KF_ERR_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return KF_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // median of 5 timed repetitions after one warm-up of a launch sequence
    auto time_it = [&](auto&& launch) {
        launch();
        float t[5];
        for (float& x : t) {
            cudaEventRecord(e0, b->stream);
            launch();
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&x, e0, e1);
        }
        std::sort(t, t + 5);
        return t[2];
    };
    // the ICP group pass at the finest level: warps per block
    float best = 1e30f;
    for (int w : {4, 8, 16}) {
        const float t = time_it([&] { launch_icp_group_batch(b->d_table, b->n, b->max_groups[0], 0, w, b->stream); });
        if (t < best) best = t, b->tuning[0] = w;
    }
    // the ray cast: tile shape x blocks per SM
    best = 1e30f;
    for (int shape = 0; shape < 3; ++shape)
        for (int per_sm = 1; per_sm <= 4; ++per_sm) {
            const float t = time_it([&] {
                launch_raycast_batch(b->d_table, b->n, total_ray_tiles(b, shape), b->f16, shape, per_sm * b->sms,
                                     b->d_tiles, b->stream);
            });
            if (t < best) best = t, b->tuning[1] = shape, b->tuning[2] = per_sm;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t e = cudaGetLastError();
    destroy_graphs(b);
    if (tuning) std::memcpy(tuning, b->tuning, sizeof(b->tuning));
    return e == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}

}  // extern "C"
