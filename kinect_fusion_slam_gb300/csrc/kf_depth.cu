// Depth ingest, vertex/normal map, bilateral filter and small utility kernels.
#include "kf_kernels.h"

namespace kf {

namespace {

__global__ void fill_nan_kernel(float* p, size_t n)
{
    const float v = qnan();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void fill_nan_half2_kernel(__half2* p, size_t n)
{
    const __half h = __ushort_as_half(0x7e00);
    const __half2 v = __halves2half2(h, h);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__device__ __forceinline__ float ingest(uint16_t raw, float dmin, float dmax)
{
    // LoadDepthData's convertTo + GetRangeDepth's inclusive cv::inRange mask
    // (system_utility.cpp:58-68, 77-85)
    const float d = (float)raw;
    return (d >= dmin && d <= dmax) ? d : 0.f;
}

// Frame start of Estimate_Sensor_Pose (sensor_pose_estimation.cu:255-259, 343), by one
// warp: T_prev^-1 = inv4(T), F = mat4(T_prev^-1, T).  The previous frame's integration
// inverted the same pose when T has not changed since, so its inverse is copied;
// otherwise the warp inverts T.
__device__ __forceinline__ void icp_frame_setup(State* st, int lane)
{
    const bool same = __all_sync(0xffffffffu, lane >= 16 || __float_as_uint(st->T[lane]) ==
                                                                __float_as_uint(st->Tinv_src[lane]));
    if (same) {
        if (lane < 16) st->Tprev_inv[lane] = st->Tinv[lane];
    } else {
        inv4_warp(st->T, st->Tprev_inv);
    }
    __syncwarp();
    if (lane < 16) {
        st->F[lane] = mat4_at(st->Tprev_inv, st->T, lane);
        st->Td[lane] = (double)st->T[lane];
    }
    if (lane == 0) st->iter = 0;
}

// raw_vertices.cu:3-51 for pixel (row, col) with depth d and its lower and right
// neighbours' depths dd, dr (read only inside the image); the mask is kept in vmap.w.
__device__ __forceinline__ void vertex_at(int row, int col, float d, float dd, float dr, float4* __restrict__ vmap,
                                          float4* __restrict__ nmap, const Camera& cam)
{
    const int H = cam.H, W = cam.W;
    const int i = row * W + col;
    float4 v = make_float4(0.f, 0.f, d, 0.f);
    float4 n = make_float4(0.f, 0.f, 0.f, 0.f);
    if (d != 0 && row != H - 1 && col != W - 1) {
        v.w = 1.f;
        if (dd != 0 && dr != 0) {
            const float* Ki = cam.Ki;
            const float X = (float)(col + 1), Y = (float)(row + 1);
            const float px = d * (Ki[0] * X + Ki[1] * Y + Ki[2]);
            const float py = d * (Ki[3] * X + Ki[4] * Y + Ki[5]);
            const float dx = dd * (Ki[0] * X + Ki[1] * (float)(row + 2) + Ki[2]);
            const float rx = dr * (Ki[0] * (float)(col + 2) + Ki[1] * Y + Ki[2]);
            const float dy = dd * (Ki[3] * X + Ki[4] * (float)(row + 2) + Ki[5]);
            const float ry = dr * (Ki[3] * (float)(col + 2) + Ki[4] * Y + Ki[5]);
            // (v_down - v) x (v_right - v)
            const float n0 = (dy - py) * (dr - d) - (dd - d) * (ry - py);
            const float n1 = (dd - d) * (rx - px) - (dx - px) * (dr - d);
            const float n2 = (dx - px) * (ry - py) - (dy - py) * (rx - px);
            const float len = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
            v.x = px;
            v.y = py;
            n = make_float4(n0 / len, n1 / len, n2 / len, 0.f);
        }
    }
    vmap[i] = v;
    nmap[i] = n;
}

// One thread per pixel (batched scenes): the depth and its neighbours from global memory.
template <bool RAW>
__device__ __forceinline__ void vertex_body(int i, const uint16_t* __restrict__ raw, float* __restrict__ depth,
                                            float4* __restrict__ vmap, float4* __restrict__ nmap, const Camera& cam,
                                            float dmin, float dmax, State* st, int init_icp, int normals)
{
    const int H = cam.H, W = cam.W;
    if (init_icp && i < 32) icp_frame_setup(st, i);
    if (i >= H * W) return;
    const int row = i / W, col = i % W;
    float d;
    if (RAW) {
        d = ingest(raw[i], dmin, dmax);
        depth[i] = d;
    } else {
        d = depth[i];
    }
    if (!normals) return;
    float dd = 0.f, dr = 0.f;
    if (d != 0 && row != H - 1 && col != W - 1) {
        const int down = (row + 1) * W + col, right = row * W + col + 1;
        dd = RAW ? ingest(raw[down], dmin, dmax) : depth[down];
        dr = RAW ? ingest(raw[right], dmin, dmax) : depth[right];
    }
    vertex_at(row, col, d, dd, dr, vmap, nmap, cam);
}

// One handle's image: 32x8-pixel tiles whose depths (ingested from the raw frame, or the
// given depth) are staged in shared memory with the row below and the column to the
// right, so each pixel's two neighbours come from the tile.  The grid's first warp also
// prepares the frame's ICP (init_icp).
constexpr int kVtx = 32, kVty = 8;

template <bool RAW>
__global__ void __launch_bounds__(kVtx* kVty) vertex_kernel(const uint16_t* __restrict__ raw, float* __restrict__ depth,
                                                            float4* __restrict__ vmap, float4* __restrict__ nmap,
                                                            Camera cam, float dmin, float dmax, State* st, int init_icp,
                                                            int normals)
{
    // the next kernel (launched with launch_pdl) may be scheduled now; it waits for this
    // one before reading anything it writes
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ float sd[kVty + 1][kVtx + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int H = cam.H, W = cam.W;
    const int col = blockIdx.x * kVtx + tx, row = blockIdx.y * kVty + ty;
    if (init_icp && blockIdx.x == 0 && blockIdx.y == 0 && ty == 0) icp_frame_setup(st, tx);
    const auto load = [&](int r, int c) { return RAW ? ingest(raw[r * W + c], dmin, dmax) : depth[r * W + c]; };
    const bool in = row < H && col < W;
    float d = 0.f;
    if (in) {
        d = load(row, col);
        if (RAW) depth[row * W + col] = d;
    }
    if (!normals) return;  // the same in every thread
    sd[ty][tx] = d;
    if (ty == kVty - 1) sd[kVty][tx] = row + 1 < H && col < W ? load(row + 1, col) : 0.f;
    if (tx == kVtx - 1) sd[ty][kVtx] = row < H && col + 1 < W ? load(row, col + 1) : 0.f;
    __syncthreads();
    if (in) vertex_at(row, col, d, sd[ty + 1][tx], sd[ty][tx + 1], vmap, nmap, cam);
}

// every scene of a batch: level 0 from the raw depth (with the ICP set-up), or level l
// from that level's depth
__global__ void __launch_bounds__(256) vertex_batch_kernel(const SceneDev* __restrict__ scenes, int level,
                                                           int init_icp)
{
    const SceneDev& d = scenes[blockIdx.y];
    const Camera& cam = d.cam[level];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cam.H * cam.W && !(init_icp && i < 32)) return;  // the first warp sets up the ICP
    if (level == 0)
        vertex_body<true>(i, d.raw, d.depth[0], d.vmap[0], d.nmap[0], cam, d.dmin, d.dmax, d.st, init_icp, 1);
    else
        vertex_body<false>(i, nullptr, d.depth[level], d.vmap[level], d.nmap[level], cam, d.dmin, d.dmax, d.st, 0, 1);
}

constexpr int kBilTx = 32, kBilTy = 8, kBilMaxR = 7;

// bilateral_filtering.cu:3-47 with the interior bound tightened to y <= H-1-r,
// x <= W-1-r so the 7x7 window never leaves the image (the reference's `<= H - r`
// reads one row/column past it); pixels outside the interior are 0, as the reference's
// zero-initialised output buffer leaves them.  In the frame loop the filter sits at the
// reference's commented-out call site (kinfu_pipeline.cpp:141-145), after the vertex map.
// That call writes bilateral_output, which nothing reads; this library instead feeds the
// result forward as if written over depth_image_next, which Estimate_Sensor_Pose reads as
// the vertices' z (kinfu_pipeline.cpp:146-160): with vmap given, its z takes the filtered
// depth too (x, y, the mask and the normals stay those of the unfiltered depth).
__global__ void __launch_bounds__(kBilTx* kBilTy) bilateral_kernel(const float* __restrict__ depth,
                                                                    float* __restrict__ out,
                                                                    const float* __restrict__ spatial, int r,
                                                                    float sigma_r, int H, int W,
                                                                    float4* __restrict__ vmap)
{
    __shared__ float tile[(kBilTy + 2 * kBilMaxR) * (kBilTx + 2 * kBilMaxR)];
    __shared__ float sw[(2 * kBilMaxR + 1) * (2 * kBilMaxR + 1)];
    const int kl = 2 * r + 1;
    const int tw = kBilTx + 2 * r, th = kBilTy + 2 * r;
    const int x0 = blockIdx.x * kBilTx - r, y0 = blockIdx.y * kBilTy - r;
    const int tid = threadIdx.y * kBilTx + threadIdx.x;
    for (int k = tid; k < kl * kl; k += kBilTx * kBilTy) sw[k] = spatial[k];
    for (int k = tid; k < tw * th; k += kBilTx * kBilTy) {
        const int gx = x0 + k % tw, gy = y0 + k / tw;
        tile[k] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? depth[gy * W + gx] : 0.f;
    }
    __syncthreads();
    const int x = blockIdx.x * kBilTx + threadIdx.x, y = blockIdx.y * kBilTy + threadIdx.y;
    if (x >= W || y >= H) return;
    float res = 0.f;
    if (y >= r && y <= H - 1 - r && x >= r && x <= W - 1 - r) {
        const float c = tile[(threadIdx.y + r) * tw + threadIdx.x + r];
        const float denom = 2 * sigma_r * sigma_r;
        float sum = 0.f;
        for (int dy = 0; dy < kl; ++dy)
            for (int dx = 0; dx < kl; ++dx) {
                float t = tile[(threadIdx.y + dy) * tw + threadIdx.x + dx] - c;
                t = expf(-(t * t) / denom);
                sum = sum + (sw[dy * kl + dx] * t + 0.000000001f);
            }
        float acc = 0.f;
        for (int dy = 0; dy < kl; ++dy)
            for (int dx = 0; dx < kl; ++dx) {
                const float v = tile[(threadIdx.y + dy) * tw + threadIdx.x + dx];
                float t = v - c;
                t = expf(-(t * t) / denom);
                const float wt = sw[dy * kl + dx] * t + 0.000000001f;
                acc = acc + (wt / sum) * v;
            }
        res = acc;
    }
    out[y * W + x] = res;
    if (vmap) reinterpret_cast<float*>(vmap + y * W + x)[2] = res;
}

// flip iff acos(c) * (180/pi) > 90 (voxel_traversal.cu:361-364, double acos).  acos is
// monotone, so over floats the predicate is "c below a threshold"; find the threshold
// with the device's own acos by bisection over the float order in [-1e-3, 1e-3].
__device__ bool flips(float c)
{
    const double angle = acos((double)c) * (180.0f / 3.141592654f);
    return angle > 90;
}

__device__ __forceinline__ int float_key(float f)
{
    const int b = __float_as_int(f);
    return b >= 0 ? b : -(b & 0x7fffffff);
}

__device__ __forceinline__ float key_float(int k) { return k >= 0 ? __int_as_float(k) : -__int_as_float(-k); }

__global__ void calibrate_kernel(State* st)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int lo = float_key(-1e-3f), hi = float_key(1e-3f);  // flips(lo) true, flips(hi) false
    for (int it = 0; it < 64 && hi - lo > 1; ++it) {
        const int mid = lo + (hi - lo) / 2;
        if (flips(key_float(mid)))
            lo = mid;
        else
            hi = mid;
    }
    st->c_flip = key_float(hi);
}

// pose back to identity, ICP bookkeeping and error flag to zero; keeps the calibrated c_flip
// and the wait limit
__global__ void state_reset_kernel(State* st)
{
    const float c_flip = st->c_flip;
    const long long wait_limit = st->wait_limit;
    __syncthreads();
    unsigned* w = reinterpret_cast<unsigned*>(st);
    for (int i = threadIdx.x; i < (int)(sizeof(State) / sizeof(unsigned)); i += blockDim.x) w[i] = 0u;
    __syncthreads();
    if (threadIdx.x < 16) {
        st->T[threadIdx.x] = (threadIdx.x % 5 == 0) ? 1.f : 0.f;
        st->Td[threadIdx.x] = (threadIdx.x % 5 == 0) ? 1.0 : 0.0;
    }
    if (threadIdx.x == 0) {
        st->c_flip = c_flip;
        st->wait_limit = wait_limit;
    }
}

// x-fastest (device) <-> z-fastest (reference) volume order
__global__ void to_zfast_kernel(const float* __restrict__ src, float* __restrict__ dst, Grid g)
{
    const size_t n = (size_t)g.dx * g.dy * g.dz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t x = i % g.dx, y = (i / g.dx) % g.dy, z = i / ((size_t)g.dx * g.dy);
        dst[(x * g.dy + y) * g.dz + z] = src[i];
    }
}

__global__ void from_zfast_kernel(const float* __restrict__ src, float* __restrict__ dst, Grid g)
{
    const size_t n = (size_t)g.dx * g.dy * g.dz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t x = i % g.dx, y = (i / g.dx) % g.dy, z = i / ((size_t)g.dx * g.dy);
        dst[i] = src[(x * g.dy + y) * g.dz + z];
    }
}

__global__ void half2_to_zfast_kernel(const __half2* __restrict__ src, float* __restrict__ tsdf,
                                      float* __restrict__ weight, Grid g)
{
    const size_t n = (size_t)g.dx * g.dy * g.dz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t x = i % g.dx, y = (i / g.dx) % g.dy, z = i / ((size_t)g.dx * g.dy);
        const float2 v = __half22float2(src[i]);
        const size_t j = (x * g.dy + y) * g.dz + z;
        tsdf[j] = v.x;
        weight[j] = v.y;
    }
}

__global__ void zfast_to_half2_kernel(const float* __restrict__ tsdf, const float* __restrict__ weight,
                                      __half2* __restrict__ dst, Grid g)
{
    const size_t n = (size_t)g.dx * g.dy * g.dz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t x = i % g.dx, y = (i / g.dx) % g.dy, z = i / ((size_t)g.dx * g.dy);
        const size_t j = (x * g.dy + y) * g.dz + z;
        dst[i] = __floats2half2_rn(tsdf[j], weight[j]);
    }
}

int grid_for(size_t n, int block)
{
    const size_t b = (n + block - 1) / block;
    return (int)(b < 152 * 32 ? (b == 0 ? 1 : b) : 152 * 32);
}

}  // namespace

void launch_fill_nan(float* p, size_t n, cudaStream_t s) { fill_nan_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n); }

void launch_fill_nan_half2(__half2* p, size_t n, cudaStream_t s)
{
    fill_nan_half2_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n);
}

void launch_vertex(const uint16_t* raw, float* depth, float4* vmap, float4* nmap, const Camera& cam, float dmin,
                   float dmax, State* st, bool init_icp, bool compute_normals, cudaStream_t s)
{
    const dim3 grid((cam.W + kVtx - 1) / kVtx, (cam.H + kVty - 1) / kVty), block(kVtx, kVty);
    if (raw)
        vertex_kernel<true><<<grid, block, 0, s>>>(raw, depth, vmap, nmap, cam, dmin, dmax, st, init_icp ? 1 : 0,
                                                   compute_normals ? 1 : 0);
    else
        vertex_kernel<false><<<grid, block, 0, s>>>(raw, depth, vmap, nmap, cam, dmin, dmax, st, init_icp ? 1 : 0,
                                                    compute_normals ? 1 : 0);
}

const void* vertex_raw_kernel_func() { return reinterpret_cast<const void*>(&vertex_kernel<true>); }

void launch_bilateral(const float* depth, float* out, const float* spatial, int r, float sigma_r, int H, int W,
                      float4* vmap, cudaStream_t s)
{
    dim3 block(kBilTx, kBilTy), grid((W + kBilTx - 1) / kBilTx, (H + kBilTy - 1) / kBilTy);
    bilateral_kernel<<<grid, block, 0, s>>>(depth, out, spatial, r, sigma_r, H, W, vmap);
}

void launch_calibrate(State* st, cudaStream_t s) { calibrate_kernel<<<1, 32, 0, s>>>(st); }

void launch_state_reset(State* st, cudaStream_t s) { state_reset_kernel<<<1, 256, 0, s>>>(st); }

void launch_to_zfast_f32(const float* src, float* dst, const Grid& g, cudaStream_t s)
{
    to_zfast_kernel<<<152 * 16, 256, 0, s>>>(src, dst, g);
}

void launch_from_zfast_f32(const float* src, float* dst, const Grid& g, cudaStream_t s)
{
    from_zfast_kernel<<<152 * 16, 256, 0, s>>>(src, dst, g);
}

void launch_half2_to_zfast(const __half2* src, float* tsdf, float* weight, const Grid& g, cudaStream_t s)
{
    half2_to_zfast_kernel<<<152 * 16, 256, 0, s>>>(src, tsdf, weight, g);
}

void launch_zfast_to_half2(const float* tsdf, const float* weight, __half2* dst, const Grid& g, cudaStream_t s)
{
    zfast_to_half2_kernel<<<152 * 16, 256, 0, s>>>(tsdf, weight, dst, g);
}

}  // namespace kf

namespace kf {
namespace {

// The predicted points with surface_prediction_z != 0 (threeD_viewer.cpp:26), packed:
// (x, y, z, pixel index as int bits) and (nx, ny, nz, 0).  One atomic per warp.
__global__ void __launch_bounds__(256) compact_cloud_kernel(const float4* __restrict__ pv,
                                                            const float4* __restrict__ pn, int n,
                                                            float4* __restrict__ out, unsigned* count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const float4 p = i < n ? pv[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool keep = i < n && p.z != 0.f;
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    unsigned base = 0;
    if (lane == 0 && mask) base = atomicAdd(count, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!keep) return;
    const unsigned k = base + __popc(mask & ((1u << lane) - 1u));
    const float4 q = pn[i];
    out[2 * k] = make_float4(p.x, p.y, p.z, __int_as_float(i));
    out[2 * k + 1] = make_float4(q.x, q.y, q.z, 0.f);
}

}  // namespace

void launch_compact_cloud(const float4* pv, const float4* pn, int n, float4* out, unsigned* count, cudaStream_t s)
{
    compact_cloud_kernel<<<(n + 255) / 256, 256, 0, s>>>(pv, pn, n, out, count);
}

}  // namespace kf

namespace kf {
namespace {

// One level of the depth pyramid: coarse (i, j) averages the nonzero depths of the fine
// 2x2 block (scan order: (2i,2j), (2i,2j+1), (2i+1,2j), (2i+1,2j+1)) that lie within
// `band` of the block's first nonzero depth -- block averaging with a depth-similarity
// test, so a block straddling an occlusion edge keeps the nearer surface instead of
// inventing a depth between the two.  Zero where the block has no depth.
__device__ __forceinline__ void pyramid_depth_at(int i, const float* __restrict__ fine, int Wf,
                                                 float* __restrict__ coarse, int Wc, float band)
{
    const int r = i / Wc, c = i % Wc;
    const float d[4] = {fine[(2 * r) * Wf + 2 * c], fine[(2 * r) * Wf + 2 * c + 1], fine[(2 * r + 1) * Wf + 2 * c],
                        fine[(2 * r + 1) * Wf + 2 * c + 1]};
    float ref = 0.f;
    for (int k = 0; k < 4 && ref == 0.f; ++k) ref = d[k];
    float sum = 0.f;
    int n = 0;
    for (int k = 0; k < 4; ++k)
        if (d[k] != 0.f && fabsf(d[k] - ref) <= band) {
            sum = sum + d[k];
            ++n;
        }
    coarse[i] = n ? sum / (float)n : 0.f;
}

// the previous frame's prediction at a coarser level: the fine pixel (2i, 2j)
__device__ __forceinline__ void pyramid_prediction_at(int i, const float4* __restrict__ pv_f,
                                                      const float4* __restrict__ pn_f, int Wf, float4* __restrict__ pv_c,
                                                      float4* __restrict__ pn_c, int Wc)
{
    const int j = (2 * (i / Wc)) * Wf + 2 * (i % Wc);
    pv_c[i] = pv_f[j];
    pn_c[i] = pn_f[j];
}

__global__ void __launch_bounds__(256) pyramid_depth_kernel(const float* __restrict__ fine, int Wf,
                                                            float* __restrict__ coarse, int Hc, int Wc, float band)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Hc * Wc) pyramid_depth_at(i, fine, Wf, coarse, Wc, band);
}

__global__ void __launch_bounds__(256) pyramid_prediction_kernel(const float4* __restrict__ pv_f,
                                                                 const float4* __restrict__ pn_f, int Wf,
                                                                 float4* __restrict__ pv_c, float4* __restrict__ pn_c,
                                                                 int Hc, int Wc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Hc * Wc) pyramid_prediction_at(i, pv_f, pn_f, Wf, pv_c, pn_c, Wc);
}

// level `level` of every scene's pyramid (depth and prediction) from level - 1
__global__ void __launch_bounds__(256) pyramid_batch_kernel(const SceneDev* __restrict__ scenes, int level)
{
    const SceneDev& d = scenes[blockIdx.y];
    const Camera& f = d.cam[level - 1];
    const Camera& c = d.cam[level];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.H * c.W) return;
    pyramid_depth_at(i, d.depth[level - 1], f.W, d.depth[level], c.W, d.band);
    pyramid_prediction_at(i, d.pv[level - 1], d.pn[level - 1], f.W, d.pv[level], d.pn[level], c.W);
}

}  // namespace

void launch_pyramid_depth(const float* fine, int Wf, float* coarse, int Hc, int Wc, float band, cudaStream_t s)
{
    pyramid_depth_kernel<<<(Hc * Wc + 255) / 256, 256, 0, s>>>(fine, Wf, coarse, Hc, Wc, band);
}

void launch_pyramid_prediction(const float4* pv_f, const float4* pn_f, int Wf, float4* pv_c, float4* pn_c, int Hc,
                               int Wc, cudaStream_t s)
{
    pyramid_prediction_kernel<<<(Hc * Wc + 255) / 256, 256, 0, s>>>(pv_f, pn_f, Wf, pv_c, pn_c, Hc, Wc);
}

void launch_pyramid_batch(const SceneDev* scenes, int n_scenes, int max_pixels, int level, cudaStream_t s)
{
    pyramid_batch_kernel<<<dim3((max_pixels + 255) / 256, n_scenes), 256, 0, s>>>(scenes, level);
}

void launch_vertex_batch(const SceneDev* scenes, int n_scenes, int max_pixels, int level, bool init_icp,
                         cudaStream_t s)
{
    vertex_batch_kernel<<<dim3((max_pixels + 255) / 256, n_scenes), 256, 0, s>>>(scenes, level, init_icp ? 1 : 0);
}

}  // namespace kf
