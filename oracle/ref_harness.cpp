/*
 * TEST INFRASTRUCTURE -- the reference itself, run on the CPU.
 *
 * oracle/build.py splices the kernel bodies of PoChang007/Kinect_Fusion_SLAM's
 * src/parallel_processing/{cuda_functions.cuh, projective_tsdf.cu, raw_vertices.cu,
 * voxel_traversal.cu, sensor_pose_estimation.cu, bilateral_filtering.cu} into
 * oracle/_ref/ref_kernels.inc (never committed) and this file drives them the way the
 * reference's host wrappers and KinfuPipeline do: each "launch" is an OpenMP loop
 * that sets blockIdx/threadIdx and calls the kernel body.  Only the pieces that live
 * in OpenCV (inverse, gemm, Cholesky, inRange) and the Sum_Array block reduction
 * (which needs __syncthreads) are restated, from ocv_restated.h and below.
 *
 * Exported as kfr_* with the same signatures as the oracle's kfo_* so the tests can
 * compare the two directly.
 */
#include "ref_shim.h"

#include <vector>

thread_local kf_ref_dim3 blockIdx, threadIdx, blockDim;
thread_local int32_t* kf_ref_hit_plane = nullptr;

#include "_ref/ref_kernels.inc"

#include "kf_oracle.h"
#include "ocv_restated.h"

namespace {

template <class Fn>
void launch(long n, Fn&& fn, long chunk = 4096)
{
#pragma omp parallel for schedule(dynamic, chunk)
    for (long i = 0; i < n; ++i) {
        blockDim = kf_ref_dim3{64, 1, 1};
        blockIdx = kf_ref_dim3{(unsigned)(i / 64), 0, 0};
        threadIdx = kf_ref_dim3{(unsigned)(i % 64), 0, 0};
        fn();
    }
}

/* voxel-centre coordinate arrays as built by KinfuPipeline's constructor,
 * kinfu_pipeline.cpp:39-58 */
struct Coords {
    std::vector<float> x, y, z;
};

Coords make_coords(const kfo_grid* g)
{
    const int L = g->dims[0], W = g->dims[1], H = g->dims[2];
    const float vd = g->voxel_size;
    Coords c;
    const size_t n = (size_t)L * W * H;
    c.x.resize(n);
    c.y.resize(n);
    c.z.resize(n);
    const int xs = g->start[0], ys = g->start[1], zs = g->start[2];
#pragma omp parallel for schedule(static)
    for (int x = xs; x < xs + L; x++)
        for (int y = ys; y < ys + W; y++)
            for (int k = zs; k < zs + H; k++) {
                const size_t i = (size_t)(x - xs) * W * H + (size_t)(y - ys) * H + (k - zs);
                c.x[i] = x * vd + vd / 2.f;
                c.y[i] = y * vd + vd / 2.f;
                c.z[i] = k * vd + vd / 2.f;
            }
    return c;
}

void make_pixel_index(int H, int W, std::vector<float>& iy, std::vector<float>& ix)
{
    iy.resize((size_t)H * W);
    ix.resize((size_t)H * W);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            iy[y * W + x] = (float)y;
            ix[y * W + x] = (float)x;
        }
}

}  // namespace

extern "C" {

void kfr_integrate(const kfo_grid* g, int H, int W, const float* depth, const float* K, const float* Ki,
                   const float* T, const float* Ti, float* tsdf, float* weight, int first)
{
    Coords c = make_coords(g);
    const long n = (long)g->dims[0] * g->dims[1] * g->dims[2];
    float Kc[9], Tc[16], Kic[9], Tic[16];
    std::memcpy(Kc, K, sizeof(Kc));
    std::memcpy(Tc, T, sizeof(Tc));
    std::memcpy(Kic, Ki, sizeof(Kic));
    std::memcpy(Tic, Ti, sizeof(Tic));
    launch(((n + 63) / 64) * 64, [&] {
        Projective_TSDF(Kc, Tc, Kic, Tic, depth, c.x.data(), c.y.data(), c.z.data(), tsdf, weight,
                        g->truncated_distance, g->sdf_minimum, g->sdf_maximum, first != 0, (float)g->dims[0],
                        (float)g->dims[1], (float)g->dims[2], H, W);
    });
}

void kfr_raycast(const kfo_grid* g, int H, int W, const float* depth, const float* Ki, const float* T,
                 const float* tsdf, float* out6, int32_t* hit)
{
    Coords c = make_coords(g);
    std::vector<float> iy, ix;
    make_pixel_index(H, W, iy, ix);
    const long HW = (long)H * W;
    for (long i = 0; i < 6 * HW; ++i) out6[i] = 0.f;
    for (long i = 0; i < HW; ++i) hit[i] = -1;
    const float vd = g->voxel_size;
    float3 vmin = make_float3((float)(g->start[0] * vd), (float)(g->start[1] * vd), (float)(g->start[2] * vd));
    float3 vmax = make_float3((float)((g->start[0] + g->dims[0]) * vd), (float)((g->start[1] + g->dims[1]) * vd),
                              (float)((g->start[2] + g->dims[2]) * vd));
    float K[9] = {0}, Tc[16], Kic[9], Ti[16] = {0};
    std::memcpy(Tc, T, sizeof(Tc));
    std::memcpy(Kic, Ki, sizeof(Kic));
    float* tsdf_rw = const_cast<float*>(tsdf);
#pragma omp parallel
    {
        kf_ref_hit_plane = hit;
#pragma omp for schedule(dynamic, 256)
        for (long i = 0; i < ((HW + 63) / 64) * 64; ++i) {
            blockDim = kf_ref_dim3{64, 1, 1};
            blockIdx = kf_ref_dim3{(unsigned)(i / 64), 0, 0};
            threadIdx = kf_ref_dim3{(unsigned)(i % 64), 0, 0};
            Voxel_Traversal(out6, out6 + HW, out6 + 2 * HW, out6 + 3 * HW, out6 + 4 * HW, out6 + 5 * HW, ix.data(),
                            iy.data(), K, Tc, Kic, Ti, depth, c.x.data(), c.y.data(), c.z.data(), tsdf_rw,
                            g->dims[0], g->dims[1], g->dims[2], g->truncated_distance, vmin, vmax, vd, H, W);
        }
        kf_ref_hit_plane = nullptr;
    }
}

void kfr_vertex_normal(int H, int W, const float* depth, const float* Ki, float* vx, float* vy, float* nx,
                       float* ny, float* nz, uint8_t* mask)
{
    std::vector<float> iy, ix;
    make_pixel_index(H, W, iy, ix);
    const long HW = (long)H * W;
    for (long i = 0; i < HW; ++i) {
        vx[i] = vy[i] = nx[i] = ny[i] = nz[i] = 0.f;
        mask[i] = 0;
    }
    launch(((HW + 63) / 64) * 64, [&] {
        Calculate_Vertices_And_Normals(depth, Ki, vx, vy, nx, ny, nz, mask, iy.data(), ix.data(), H, W);
    });
}

/* ICP kernel + Sum_Array tree per 64-thread block + serial host sum
 * (sensor_pose_estimation.cu:349-387) */
int kfr_icp_associate(int H, int W, const float* K, const float* F, const float* T, const float* cur6,
                      const uint8_t* mask, const float* pred6, int32_t* pair, float* sums42)
{
    const long HW = (long)H * W;
    std::vector<float> right(6 * HW, 0.f), left(36 * HW, 0.f);
    float Kc[9], Fc[16], Tc[16], Ti[16] = {0};
    std::memcpy(Kc, K, sizeof(Kc));
    std::memcpy(Fc, F, sizeof(Fc));
    std::memcpy(Tc, T, sizeof(Tc));
    launch(((HW + 63) / 64) * 64, [&] {
        ICP(cur6, cur6 + HW, cur6 + 2 * HW, cur6 + 3 * HW, cur6 + 4 * HW, cur6 + 5 * HW, pred6, pred6 + HW,
            pred6 + 2 * HW, pred6 + 3 * HW, pred6 + 4 * HW, pred6 + 5 * HW, Kc, Ti, Tc, Fc, right.data(),
            left.data(), mask, H, W);
    });
    int ncorr = 0;
    for (long i = 0; i < HW; ++i) {
        bool any = false;
        for (int k = 0; k < 6 && !any; ++k) any = right[k * HW + i] != 0.f;
        for (int k = 0; k < 36 && !any; ++k) any = left[k * HW + i] != 0.f;
        if (pair) pair[i] = any ? 1 : 0; /* the reference has no pairing output: 1 marks a non-zero row */
        ncorr += any;
    }
    const int nblocks = (int)((HW + 63) / 64);
    std::vector<float> part(nblocks);
    for (int k = 0; k < 42; ++k) {
        const float* plane = k < 6 ? right.data() + k * HW : left.data() + (k - 6) * HW;
        for (int b = 0; b < nblocks; ++b) {
            float s[64];
            /* a last, partial block is padded with zeros, as the oracle does (the
             * reference runs 640x480 = 4800 full blocks only) */
            for (int t = 0; t < 64; ++t) s[t] = (long)b * 64 + t < HW ? plane[b * 64 + t] : 0.f;
            for (int st = 32; st > 0; st >>= 1)
                for (int t = 0; t < st; ++t) s[t] += s[t + st];
            part[b] = s[0];
        }
        float acc = 0.0f;
        for (int b = 0; b < nblocks; ++b) acc += part[b];
        sums42[k] = acc;
    }
    return ncorr;
}

void kfr_estimate_pose(int H, int W, const float* K, float* T, const float* cur6, const uint8_t* mask,
                       const float* pred6, int iters, float* sums_log, float* pose_log)
{
    float Tinv[16], R[16], F[16];
    ocv_inv4(T, Tinv);
    std::memcpy(R, T, sizeof(R));
    for (int it = 0; it < iters; ++it) {
        ocv_matmul4(Tinv, R, F);
        float s[42];
        kfr_icp_associate(H, W, K, F, R, cur6, mask, pred6, nullptr, s);
        if (sums_log) std::memcpy(sums_log + it * 42, s, sizeof(s));
        float A[36], b[6];
        std::memcpy(A, s + 6, sizeof(A));
        std::memcpy(b, s, sizeof(b));
        ocv_cholesky6(A, b);
        const float inc[16] = {1.0f, b[2], -b[1], b[3], -b[2], 1.0f, b[0], b[4],
                               b[1], -b[0], 1.0f, b[5], 0.0f, 0.0f, 0.0f, 1.0f};
        ocv_matmul4(inc, R, R);
        if (pose_log) std::memcpy(pose_log + it * 16, R, sizeof(R));
    }
    std::memcpy(T, R, sizeof(R));
}

/* the reference kernel reads one row/column past the image at its upper bound; the
 * input is padded with a zero row so the read stays inside the buffer */
void kfr_bilateral(int H, int W, const float* depth, const float* spatial, int r, float sigma_r, float* out)
{
    std::vector<float> iy, ix;
    make_pixel_index(H, W, iy, ix);
    const long HW = (long)H * W;
    std::vector<float> padded((size_t)(H + 2) * W, 0.f);
    std::memcpy(padded.data(), depth, sizeof(float) * HW);
    for (long i = 0; i < HW; ++i) out[i] = 0.f;
    launch(((HW + 63) / 64) * 64, [&] {
        Bilateral_Filtering(padded.data(), out, spatial, iy.data(), ix.data(), r, sigma_r, H, W);
    }, 256);
}

/* ---- KinfuPipeline frame loop with the reference kernels ---- */
struct kfr_pipeline {
    int H, W;
    float min_depth, max_depth;
    kfo_grid g;
    float K[9], T[16];
    std::vector<float> tsdf, weight, depth, cur6, pred6;
    std::vector<uint8_t> mask;
    std::vector<int32_t> hit;
};

kfr_pipeline* kfr_create(int H, int W, float min_depth, float max_depth, const kfo_grid* g, const float* K)
{
    kfr_pipeline* p = new kfr_pipeline;
    p->H = H;
    p->W = W;
    p->min_depth = min_depth;
    p->max_depth = max_depth;
    p->g = *g;
    std::memcpy(p->K, K, sizeof(p->K));
    for (int i = 0; i < 16; ++i) p->T[i] = (i % 5 == 0) ? 1.f : 0.f;
    const size_t n = (size_t)g->dims[0] * g->dims[1] * g->dims[2];
    p->tsdf.assign(n, NAN);
    p->weight.assign(n, NAN);
    p->depth.assign((size_t)H * W, 0.f);
    p->cur6.assign((size_t)6 * H * W, 0.f);
    p->pred6.assign((size_t)6 * H * W, 0.f);
    p->mask.assign((size_t)H * W, 0);
    p->hit.assign((size_t)H * W, -1);
    return p;
}

void kfr_destroy(kfr_pipeline* p) { delete p; }

static void ingest(kfr_pipeline* p, const uint16_t* raw)
{
    for (long i = 0; i < (long)p->H * p->W; ++i) {
        const float d = (float)raw[i];
        p->depth[i] = (d >= p->min_depth && d <= p->max_depth) ? d : 0.f;
    }
}

void kfr_initial(kfr_pipeline* p, const uint16_t* raw)
{
    ingest(p, raw);
    float Ki[9], Ti[16];
    ocv_inv3(p->K, Ki);
    ocv_inv4(p->T, Ti);
    kfr_integrate(&p->g, p->H, p->W, p->depth.data(), p->K, Ki, p->T, Ti, p->tsdf.data(), p->weight.data(), 1);
    kfr_raycast(&p->g, p->H, p->W, p->depth.data(), Ki, p->T, p->tsdf.data(), p->pred6.data(), p->hit.data());
}

void kfr_incoming(kfr_pipeline* p, const uint16_t* raw, int icp_iters)
{
    const int H = p->H, W = p->W;
    const long HW = (long)H * W;
    ingest(p, raw);
    float Ki[9];
    ocv_inv3(p->K, Ki);
    float* c = p->cur6.data();
    kfr_vertex_normal(H, W, p->depth.data(), Ki, c, c + HW, c + 3 * HW, c + 4 * HW, c + 5 * HW, p->mask.data());
    std::memcpy(c + 2 * HW, p->depth.data(), sizeof(float) * HW);
    kfr_estimate_pose(H, W, p->K, p->T, c, p->mask.data(), p->pred6.data(), icp_iters, nullptr, nullptr);
    float Ti[16];
    ocv_inv4(p->T, Ti);
    kfr_integrate(&p->g, H, W, p->depth.data(), p->K, Ki, p->T, Ti, p->tsdf.data(), p->weight.data(), 0);
    kfr_raycast(&p->g, H, W, p->depth.data(), Ki, p->T, p->tsdf.data(), p->pred6.data(), p->hit.data());
}

void kfr_get_pose(const kfr_pipeline* p, float* T) { std::memcpy(T, p->T, sizeof(p->T)); }

void kfr_get_prediction(const kfr_pipeline* p, float* out6, int32_t* hit)
{
    if (out6) std::memcpy(out6, p->pred6.data(), sizeof(float) * p->pred6.size());
    if (hit) std::memcpy(hit, p->hit.data(), sizeof(int32_t) * p->hit.size());
}

void kfr_get_volume(const kfr_pipeline* p, float* tsdf, float* weight)
{
    if (tsdf) std::memcpy(tsdf, p->tsdf.data(), sizeof(float) * p->tsdf.size());
    if (weight) std::memcpy(weight, p->weight.data(), sizeof(float) * p->weight.size());
}

}  // extern "C"
