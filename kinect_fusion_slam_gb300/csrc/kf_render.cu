// The differentiation form: a trilinear ray-cast renderer of a TSDF and its adjoint.
//
// Forward, per pixel (u, v) (1-based, the reference's convention): the ray
// x(t) = o + t r with o the camera centre and r = R K^-1 [u, v, 1] (so t is the camera-z
// depth) is marched from t_near in steps of `step`; at each sample the TSDF is
// interpolated trilinearly from the 8 voxel centres around it (a sample with a corner
// outside the grid or unobserved (NaN) is invalid).  The first pair of consecutive
// valid samples with f_a > 0 >= f_b brackets the surface; the rendered depth is the
// linear zero crossing t* = t_a + (t_b - t_a) f_a / (f_a - f_b) and the normal is the
// normalised trilinear gradient at x* = x(t*).  Pixels without a bracket render 0.
//
// Adjoint: the backward kernel recomputes each ray's march (nothing is stored) and
// applies the chain rule to exactly the function the forward computes:
//   t* depends on f_a and f_b, which depend on their 8 voxels (weights w_c) and on the
//   pose through the sample positions; the normal n = g/|g| depends on the 8 voxels of
//   x*'s cell (through the weight gradients) and on x* (through the trilinear Hessian).
// With the pose perturbed on the left, T(xi) = exp(xi^) T, xi = (omega, tau) in world
// coordinates, a point x on a ray moves by omega x x + tau, so a sampled value changes
// by d f = (x x grad f) . omega + grad f . tau.  Voxel gradients are scattered with
// warp-aggregated atomics (lanes that hit the same voxel add their contributions first);
// the pose gradient is reduced per block and added atomically.
#include <cmath>
#include <cstdint>
#include <vector>

#include "kinfu_gb300.h"
#include "kf_kernels.h"
#include "kf_math.cuh"

namespace kf {
namespace {

struct RenderGeom {
    int H, W;
    float Ki[9];
    float R[9];
    float3 o;
    int dx, dy, dz;
    float gx0, gy0, gz0;  // continuous index of world 0: -(start + 0.5)
    float inv_vd;
    float t_near, t_far, step;
    int max_steps;
    float max_residual;  // Gauss-Newton gate (infinity = none)
    float huber;         // Huber threshold of the normal equations (0 = plain least squares)
};

struct Corner8 {
    int base;       // linear index of the (i0, j0, k0) corner, x-fastest
    float fx, fy, fz;
    float c[8];     // c[(k << 2) | (j << 1) | i]
};

// trilinear sample at world point x; false if a corner is outside the grid or NaN
__device__ __forceinline__ bool fetch(const float* __restrict__ V, const RenderGeom& g, float3 x, Corner8& s)
{
    const float gx = fmaf(x.x, g.inv_vd, g.gx0), gy = fmaf(x.y, g.inv_vd, g.gy0), gz = fmaf(x.z, g.inv_vd, g.gz0);
    const float ix = floorf(gx), iy = floorf(gy), iz = floorf(gz);
    if (!(ix >= 0.f && iy >= 0.f && iz >= 0.f && ix <= (float)(g.dx - 2) && iy <= (float)(g.dy - 2) &&
          iz <= (float)(g.dz - 2)))
        return false;
    const int i = (int)ix, j = (int)iy, k = (int)iz;
    s.fx = gx - ix;
    s.fy = gy - iy;
    s.fz = gz - iz;
    const int sy = g.dx, sz = g.dx * g.dy;
    s.base = (k * g.dy + j) * g.dx + i;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float v = __ldg(V + s.base + (q & 1) + ((q >> 1) & 1) * sy + (q >> 2) * sz);
        s.c[q] = v;
        ok = ok && !isnan(v);
    }
    return ok;
}

__device__ __forceinline__ float weight(const Corner8& s, int q)
{
    return ((q & 1) ? s.fx : 1.f - s.fx) * (((q >> 1) & 1) ? s.fy : 1.f - s.fy) * ((q >> 2) ? s.fz : 1.f - s.fz);
}

__device__ __forceinline__ float value(const Corner8& s)
{
    float f = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) f += weight(s, q) * s.c[q];
    return f;
}

// world-space gradient of the trilinear interpolant
__device__ __forceinline__ float3 gradient(const Corner8& s, float inv_vd)
{
    const float ax = 1.f - s.fx, ay = 1.f - s.fy, az = 1.f - s.fz;
    const float* c = s.c;
    const float dfx = ((c[1] - c[0]) * ay + (c[3] - c[2]) * s.fy) * az + ((c[5] - c[4]) * ay + (c[7] - c[6]) * s.fy) * s.fz;
    const float dfy = ((c[2] - c[0]) * ax + (c[3] - c[1]) * s.fx) * az + ((c[6] - c[4]) * ax + (c[7] - c[5]) * s.fx) * s.fz;
    const float dfz = ((c[4] - c[0]) * ax + (c[5] - c[1]) * s.fx) * ay + ((c[6] - c[2]) * ax + (c[7] - c[3]) * s.fx) * s.fy;
    return make_float3(dfx * inv_vd, dfy * inv_vd, dfz * inv_vd);
}

// the trilinear Hessian's off-diagonal entries (world units): xy, xz, yz
__device__ __forceinline__ float3 hessian(const Corner8& s, float inv_vd)
{
    const float* c = s.c;
    const float i2 = inv_vd * inv_vd;
    const float hxy = ((c[3] - c[2] - c[1] + c[0]) * (1.f - s.fz) + (c[7] - c[6] - c[5] + c[4]) * s.fz) * i2;
    const float hxz = ((c[5] - c[4] - c[1] + c[0]) * (1.f - s.fy) + (c[7] - c[6] - c[3] + c[2]) * s.fy) * i2;
    const float hyz = ((c[6] - c[4] - c[2] + c[0]) * (1.f - s.fx) + (c[7] - c[5] - c[3] + c[1]) * s.fx) * i2;
    return make_float3(hxy, hxz, hyz);
}

__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 scale3(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct Ray {
    float3 o, r;
};

__device__ __forceinline__ Ray pixel_ray(const RenderGeom& g, int i)
{
    const float X = (float)(i % g.W) + 1.f, Y = (float)(i / g.W) + 1.f;
    const float3 d = make_float3(g.Ki[0] * X + g.Ki[1] * Y + g.Ki[2], g.Ki[3] * X + g.Ki[4] * Y + g.Ki[5],
                                 g.Ki[6] * X + g.Ki[7] * Y + g.Ki[8]);
    const float3 r = make_float3(g.R[0] * d.x + g.R[1] * d.y + g.R[2] * d.z, g.R[3] * d.x + g.R[4] * d.y + g.R[5] * d.z,
                                 g.R[6] * d.x + g.R[7] * d.y + g.R[8] * d.z);
    return Ray{g.o, r};
}

struct Hit {
    float ta, tb, fa, fb;  // bracket: the samples at ta and tb (one step apart)
    Corner8 a, b;
};

// the march shared by the forward and the adjoint (identical arithmetic)
__device__ __forceinline__ bool march(const float* __restrict__ V, const RenderGeom& g, const Ray& ray, Hit& hit)
{
    float t = g.t_near, prev_t = 0.f, prev_f = 0.f;
    bool prev_ok = false;
    Corner8 prev;
    for (int k = 0; k < g.max_steps && t <= g.t_far; ++k) {
        Corner8 s;
        const float3 x = add3(ray.o, scale3(ray.r, t));
        const bool ok = fetch(V, g, x, s);
        const float f = ok ? value(s) : 0.f;
        if (ok && prev_ok && prev_f > 0.f && f <= 0.f) {
            hit.ta = prev_t;
            hit.tb = t;
            hit.fa = prev_f;
            hit.fb = f;
            hit.a = prev;
            hit.b = s;
            return true;
        }
        prev_ok = ok;
        prev_f = f;
        prev_t = t;
        prev = s;
        t += g.step;
    }
    return false;
}

__global__ void __launch_bounds__(256) render_kernel(const float* __restrict__ V, RenderGeom g, float* __restrict__ depth,
                                                     float* __restrict__ normal)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.H * g.W) return;
    const Ray ray = pixel_ray(g, i);
    Hit h;
    float d = 0.f;
    float3 n = make_float3(0.f, 0.f, 0.f);
    if (march(V, g, ray, h)) {
        const float s = h.fa / (h.fa - h.fb);
        const float ts = h.ta + (h.tb - h.ta) * s;
        d = ts;
        Corner8 c;
        if (fetch(V, g, add3(ray.o, scale3(ray.r, ts)), c)) {
            const float3 gr = gradient(c, g.inv_vd);
            const float len = sqrtf(dot3(gr, gr));
            if (len > 0.f) n = scale3(gr, 1.f / len);
        }
    }
    if (depth) depth[i] = d;
    if (normal) {
        normal[3 * i] = n.x;
        normal[3 * i + 1] = n.y;
        normal[3 * i + 2] = n.z;
    }
}

// adds v to V[addr] once per distinct address in the warp (all lanes call; addr < 0 = none)
__device__ __forceinline__ void warp_aggregated_add(float* grad, int addr, float v)
{
    const unsigned full = 0xffffffffu;
    const unsigned group = __match_any_sync(full, addr);
    float sum = 0.f;
#pragma unroll 4
    for (int src = 0; src < 32; ++src) {
        const float o = __shfl_sync(full, v, src);
        if ((group >> src) & 1u) sum += o;
    }
    const int lane = threadIdx.x & 31;
    if (addr >= 0 && lane == __ffs(group) - 1) atomicAdd(grad + addr, sum);
}

__device__ __forceinline__ void corner_adds(float* grad, const RenderGeom& g, const Corner8& s, bool valid, float scale)
{
    const int sy = g.dx, sz = g.dx * g.dy;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int addr = valid ? s.base + (q & 1) + ((q >> 1) & 1) * sy + (q >> 2) * sz : -1;
        warp_aggregated_add(grad, addr, valid ? scale * weight(s, q) : 0.f);
    }
}

// d f / d xi at point x with world gradient gr: (x cross gr, gr)
__device__ __forceinline__ void pose_row(float3 x, float3 gr, float (&j)[6])
{
    const float3 w = cross3(x, gr);
    j[0] = w.x;
    j[1] = w.y;
    j[2] = w.z;
    j[3] = gr.x;
    j[4] = gr.y;
    j[5] = gr.z;
}

// MODE 0: adjoint (grad_tsdf, grad_pose).  MODE 1: Gauss-Newton sums of the depth
// residual D - measured over pixels with both: J^T J (21, upper triangle row by row),
// J^T r (6), count, sum r^2 -- per block into partials[blockIdx.x * 29 + k].
template <int MODE>
__global__ void __launch_bounds__(256) render_adjoint_kernel(const float* __restrict__ V, RenderGeom g,
                                                             const float* __restrict__ grad_depth,
                                                             const float* __restrict__ grad_normal,
                                                             float* __restrict__ grad_tsdf, float* __restrict__ grad_pose,
                                                             const float* __restrict__ measured,
                                                             float* __restrict__ partials)
{
    constexpr int kVals = MODE == 0 ? 6 : 29;
    __shared__ float red[8][kVals];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float acc[kVals];
#pragma unroll
    for (int k = 0; k < kVals; ++k) acc[k] = 0.f;

    Hit h;
    bool hit = false;
    Ray ray{};
    if (i < g.H * g.W) {
        ray = pixel_ray(g, i);
        hit = march(V, g, ray, h);
    }
    float gD = 0.f;
    float3 gN = make_float3(0.f, 0.f, 0.f);
    if (hit && MODE == 0) {
        gD = grad_depth ? grad_depth[i] : 0.f;
        if (grad_normal) gN = make_float3(grad_normal[3 * i], grad_normal[3 * i + 1], grad_normal[3 * i + 2]);
    }
    float dt_dfa = 0.f, dt_dfb = 0.f, total_t = 0.f;
    float3 ts_x = make_float3(0.f, 0.f, 0.f), hgn = make_float3(0.f, 0.f, 0.f), gn = hgn;
    Corner8 c{};
    bool nvalid = false;
    if (hit) {
        const float den = h.fa - h.fb, dt = h.tb - h.ta;
        const float s = h.fa / den;
        const float ts = h.ta + dt * s;
        dt_dfa = dt * (-h.fb) / (den * den);
        dt_dfb = dt * h.fa / (den * den);
        ts_x = add3(ray.o, scale3(ray.r, ts));
        total_t = gD;
        if (MODE == 0 && fetch(V, g, ts_x, c)) {
            const float3 gr = gradient(c, g.inv_vd);
            const float len = sqrtf(dot3(gr, gr));
            if (len > 0.f) {
                nvalid = true;
                const float3 n = scale3(gr, 1.f / len);
                // gn = (I - n n^T) gN / |g|
                gn = scale3(add3(gN, scale3(n, -dot3(n, gN))), 1.f / len);
                const float3 hs = hessian(c, g.inv_vd);  // symmetric, zero diagonal
                hgn = make_float3(hs.x * gn.y + hs.y * gn.z, hs.x * gn.x + hs.z * gn.z, hs.y * gn.x + hs.z * gn.y);
                total_t += dot3(hgn, ray.r);
            }
        }
        // dt*/dxi from the two bracketing samples
        float ja[6], jb[6];
        const float3 xa = add3(ray.o, scale3(ray.r, h.ta)), xb = add3(ray.o, scale3(ray.r, h.tb));
        pose_row(xa, gradient(h.a, g.inv_vd), ja);
        pose_row(xb, gradient(h.b, g.inv_vd), jb);
        float jt[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) jt[k] = dt_dfa * ja[k] + dt_dfb * jb[k];
        if (MODE == 0) {
            float jx[6];
            pose_row(ts_x, hgn, jx);  // zero when the normal is not differentiable here
#pragma unroll
            for (int k = 0; k < 6; ++k) acc[k] = total_t * jt[k] + jx[k];
        } else {
            const float dm = measured[i];
            const float r = ts - dm;
            if (dm > 0.f && !(fabsf(r) > g.max_residual)) {
                // Huber: weight min(1, delta / |r|) (iteratively reweighted least squares),
                // so w r = clamp(r, -delta, delta) is the loss's derivative; the loss term
                // is 2 rho(r) = r^2 inside the threshold, 2 delta |r| - delta^2 outside
                const float ar = fabsf(r);
                const bool out = g.huber > 0.f && ar > g.huber;
                const float w = out ? g.huber / ar : 1.f;
                int q = 0;
#pragma unroll
                for (int a = 0; a < 6; ++a)
#pragma unroll
                    for (int b = a; b < 6; ++b) acc[q++] = w * (jt[a] * jt[b]);
#pragma unroll
                for (int a = 0; a < 6; ++a) acc[21 + a] = jt[a] * (w * r);
                acc[27] = 1.f;
                acc[28] = out ? g.huber * (2.f * ar - g.huber) : r * r;
            }
        }
    }
    if (MODE == 0 && grad_tsdf) {
        // voxel gradients: the bracket's samples through t*, x*'s cell through the normal
        corner_adds(grad_tsdf, g, h.a, hit, total_t * dt_dfa);
        corner_adds(grad_tsdf, g, h.b, hit, total_t * dt_dfb);
        const int sy = g.dx, sz = g.dx * g.dy;
        const float ax = 1.f - c.fx, ay = 1.f - c.fy, az = 1.f - c.fz;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            // gradient of corner q's weight with respect to x*, world units
            const float wx = (q & 1) ? c.fx : ax, wy = ((q >> 1) & 1) ? c.fy : ay, wz = (q >> 2) ? c.fz : az;
            const float sx = (q & 1) ? 1.f : -1.f, sy1 = ((q >> 1) & 1) ? 1.f : -1.f, sz1 = (q >> 2) ? 1.f : -1.f;
            const float3 dw = make_float3(sx * wy * wz * g.inv_vd, sy1 * wx * wz * g.inv_vd, sz1 * wx * wy * g.inv_vd);
            const bool on = hit && nvalid;
            const int addr = on ? c.base + (q & 1) + ((q >> 1) & 1) * sy + (q >> 2) * sz : -1;
            warp_aggregated_add(grad_tsdf, addr, on ? dot3(gn, dw) : 0.f);
        }
    }
    // block reduction of the pose terms (or the normal-equation sums)
#pragma unroll
    for (int k = 0; k < kVals; ++k) {
        float v = acc[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kVals) {
        float v = 0.f;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) v += red[w][threadIdx.x];
        if (MODE == 0) {
            if (grad_pose) atomicAdd(grad_pose + threadIdx.x, v);
        } else {
            partials[(size_t)blockIdx.x * kVals + threadIdx.x] = v;
        }
    }
}

}  // namespace

}  // namespace kf

namespace {

bool make_geom(const kf_render_desc* d, const float T[16], kf::RenderGeom& g)
{
    if (!d || !T || d->height <= 0 || d->width <= 0 || !(d->fx > 0) || !(d->fy > 0) || !(d->voxel_size > 0) ||
        !(d->step > 0) || !(d->t_far > d->t_near) || d->dims[0] < 2 || d->dims[1] < 2 || d->dims[2] < 2)
        return false;
    if ((long long)d->dims[0] * d->dims[1] * d->dims[2] >= (1LL << 31)) return false;
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(T[k])) return false;
    g.H = d->height;
    g.W = d->width;
    const float K[9] = {d->fx, 0.f, d->cx, 0.f, d->fy, d->cy, 0.f, 0.f, 1.f};
    kf::inv3(K, g.Ki);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) g.R[r * 3 + c] = T[r * 4 + c];
    g.o = make_float3(T[3], T[7], T[11]);
    g.dx = d->dims[0];
    g.dy = d->dims[1];
    g.dz = d->dims[2];
    g.inv_vd = 1.f / d->voxel_size;
    g.gx0 = -((float)d->grid_start[0] + 0.5f);
    g.gy0 = -((float)d->grid_start[1] + 0.5f);
    g.gz0 = -((float)d->grid_start[2] + 0.5f);
    g.t_near = d->t_near;
    g.t_far = d->t_far;
    g.step = d->step;
    const double steps = std::ceil(((double)d->t_far - d->t_near) / d->step) + 1.0;
    g.max_steps = steps > 1e6 ? 1000000 : (int)steps;
    g.max_residual = INFINITY;
    g.huber = 0.f;
    return true;
}

}  // namespace

extern "C" kf_status kf_render_trilinear(const kf_render_desc* d, const float* tsdf, const float T[16], float* depth,
                                         float* normal, void* stream)
{
    kf::RenderGeom g;
    if (!tsdf || !make_geom(d, T, g)) return KF_ERR_INVALID_ARGUMENT;
    const int n = g.H * g.W;
    kf::render_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(tsdf, g, depth, normal);
    return cudaGetLastError() == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}

extern "C" kf_status kf_render_trilinear_backward(const kf_render_desc* d, const float* tsdf, const float T[16],
                                                  const float* grad_depth, const float* grad_normal,
                                                  float* grad_tsdf, float* grad_pose, void* stream)
{
    kf::RenderGeom g;
    if (!tsdf || !make_geom(d, T, g)) return KF_ERR_INVALID_ARGUMENT;
    const int n = g.H * g.W;
    kf::render_adjoint_kernel<0><<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        tsdf, g, grad_depth, grad_normal, grad_tsdf, grad_pose, nullptr, nullptr);
    return cudaGetLastError() == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}

extern "C" kf_status kf_render_depth_normal_equations(const kf_render_desc* d, const float* tsdf, const float T[16],
                                                      const float* measured_depth, float max_residual, double sums[29],
                                                      void* stream)
{
    return kf_render_depth_normal_equations_huber(d, tsdf, T, measured_depth, max_residual, 0.f, sums, stream);
}

extern "C" kf_status kf_render_depth_normal_equations_huber(const kf_render_desc* d, const float* tsdf,
                                                            const float T[16], const float* measured_depth,
                                                            float max_residual, float huber_delta, double sums[29],
                                                            void* stream)
{
    kf::RenderGeom g;
    if (!tsdf || !measured_depth || !sums || !make_geom(d, T, g) || std::isnan(max_residual) ||
        !(huber_delta >= 0.f))
        return KF_ERR_INVALID_ARGUMENT;
    g.max_residual = max_residual > 0.f ? max_residual : INFINITY;
    g.huber = huber_delta;
    const int n = g.H * g.W, blocks = (n + 255) / 256;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* partials = nullptr;
    if (cudaMallocAsync((void**)&partials, sizeof(float) * 29 * (size_t)blocks, s) != cudaSuccess) return KF_ERR_CUDA;
    kf::render_adjoint_kernel<1><<<blocks, 256, 0, s>>>(tsdf, g, nullptr, nullptr, nullptr, nullptr, measured_depth,
                                                        partials);
    std::vector<float> h((size_t)29 * blocks);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), partials, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(partials, s);
    if (e != cudaSuccess) return KF_ERR_CUDA;
    for (int k = 0; k < 29; ++k) sums[k] = 0.0;
    for (int b = 0; b < blocks; ++b)
        for (int k = 0; k < 29; ++k) sums[k] += (double)h[(size_t)b * 29 + k];
    return KF_OK;
}
