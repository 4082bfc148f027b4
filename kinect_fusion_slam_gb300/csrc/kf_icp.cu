// Projective point-to-plane ICP: association, one-pass reduction of the 6x6 normal
// equations and the on-device solve (sensor_pose_estimation.cu:7-136, 247-436).
//
// One launch per iteration.  Every thread associates its pixels and accumulates the
// 27 distinct sums of the reference's 42 planes (6 of a*b, the upper triangle of
// a a^T; the reference's A is exactly symmetric because a_r*a_s == a_s*a_r and both
// planes are summed in the same order) plus a correspondence count in registers; the
// block reduces them with warp shuffles and shared memory and writes one partial; the
// last block to finish (ticket counter) reduces the partials in a fixed order, solves
// the system like cv::Cholesky, forms the small-angle increment and updates the pose
// in device memory.  The reduction order differs from the reference's 64-wide tree +
// serial host sum, so the sums agree to float rounding, not bit for bit.
#include <cmath>
#include <cstddef>

#include "kf_kernels.h"
#include "kf_launch.cuh"
#include "kf_solve.cuh"

namespace kf {

namespace {

constexpr int kIcpBlock = 256;
constexpr int kIcpMaxBlocks = 152 * 4;

struct TwoSum {
    float hi, lo;
};

// Knuth's two-sum: hi + lo == a + b exactly (no FMA contraction in this file)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <bool PRECISE>
struct Acc {
    float hi[kIcpVals];
    float lo[PRECISE ? kIcpVals : 1];

    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int k = 0; k < kIcpVals; ++k) hi[k] = 0.f;
        if (PRECISE) {
#pragma unroll
            for (int k = 0; k < kIcpVals; ++k) lo[PRECISE ? k : 0] = 0.f;
        }
    }
    __device__ __forceinline__ void add(int k, float v)
    {
        if (PRECISE) {
            float s, e;
            two_sum(hi[k], v, s, e);
            hi[k] = s;
            lo[PRECISE ? k : 0] += e;
        } else {
            hi[k] += v;
        }
    }
    __device__ __forceinline__ void add_pair(int k, float h, float l)
    {
        if (PRECISE) {
            float s, e;
            two_sum(hi[k], h, s, e);
            hi[k] = s;
            lo[PRECISE ? k : 0] += e + l;
        } else {
            hi[k] += h;
        }
    }
};

// sensor_pose_estimation.cu:20-48, first half: the vertex (vmap.w holds the vertex mask),
// its projection through F and K (the reference projects through K although its kernel
// argument is named dev_inv_cam_intrinsic: the launch at :353 passes dev_cam_intrinsic)
// and, when it lands in the image, the matched pixel j and the vertex in world g
__device__ __forceinline__ bool assoc_project(float4 v, const Camera& cam, const float* F, const float* T, float3& g,
                                              int& j)
{
    if (!(v.z != 0 && v.w != 0)) return false;
    const float3 p3 = make_float3(v.x, v.y, v.z);
    const float3 c = xform(F, p3);
    const float3 p = mul3(cam.K, c);
    const int u = (int)roundf(p.x / p.z);
    const int vv = (int)roundf(p.y / p.z);
    if (!(u > 0 && u <= cam.W && vv > 0 && vv <= cam.H)) return false;
    g = xform(T, p3);
    j = (vv - 1) * cam.W + (u - 1);
    return true;
}

// second half (:44-131): the distance and normal-angle gates against the prediction
// (q, m) at j, then the row a and residual b
__device__ __forceinline__ bool assoc_finish(float3 g, float4 n, float4 q, float4 m, const float* T, float dist_th,
                                             float ang_th, float (&a)[6], float& b)
{
    const float3 dd = make_float3(g.x - q.x, g.y - q.y, g.z - q.z);
    const float dist = sqrtf(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
    if (!(dist <= dist_th && dist >= 0.0f)) return false;
    const float3 un = normalized(make_float3(T[0] * n.x + T[1] * n.y + T[2] * n.z, T[4] * n.x + T[5] * n.y + T[6] * n.z,
                                             T[8] * n.x + T[9] * n.y + T[10] * n.z));
    const float3 va = normalized(make_float3(m.x, m.y, m.z));
    const float ct = un.x * va.x + un.y * va.y + un.z * va.z;
    const float angle = acosf(ct) * (180.0f / 3.141592654f);
    if (!(angle <= ang_th && angle >= 0.0f)) return false;
    a[0] = g.z * m.y + (-g.y * m.z);
    a[1] = -g.z * m.x + (g.x * m.z);
    a[2] = g.y * m.x + (-g.x * m.y);
    a[3] = m.x;
    a[4] = m.y;
    a[5] = m.z;
    b = m.x * (q.x - g.x) + m.y * (q.y - g.y) + m.z * (q.z - g.z);
    return true;
}

__device__ __forceinline__ bool associate(int i, const float4* __restrict__ vmap, const float4* __restrict__ nmap,
                                          const float4* __restrict__ pv, const float4* __restrict__ pn,
                                          const Camera& cam, const float* F, const float* T, float dist_th,
                                          float ang_th, float (&a)[6], float& b, int& j)
{
    float3 g;
    if (!assoc_project(vmap[i], cam, F, T, g, j)) return false;
    return assoc_finish(g, nmap[i], pv[j], pn[j], T, dist_th, ang_th, a, b);
}

// The same for a lane's two pixels of a 64-pixel group (i and i + 32), arranged so
// that each round of loads is issued for both pixels before either is used -- the
// vertices and normals together, then both matched predictions -- which turns six
// dependent L2 round trips into two.  The arithmetic is associate()'s, operation for
// operation; only independent loads move.  load_pair is the first round of loads
// (the lane's two vertices and normals, zero past the image), associate_pair_from the
// rest.
__device__ __forceinline__ void load_pair(int i0, int n, const float4* __restrict__ vmap,
                                          const float4* __restrict__ nmap, float4 (&v)[2], float4 (&nn)[2])
{
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = i0 + 32 * h;
        v[h] = i < n ? vmap[i] : zero;
        nn[h] = i < n ? nmap[i] : zero;
    }
}

__device__ __forceinline__ void associate_pair_from(const float4 (&v)[2], const float4 (&nn)[2],
                                                    const float4* __restrict__ pv, const float4* __restrict__ pn,
                                                    const Camera& cam, const float* F, const float* T, float dist_th,
                                                    float ang_th, bool (&ok)[2], float (&a)[2][6], float (&b)[2],
                                                    int (&j)[2])
{
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 g[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        j[h] = -1;
        ok[h] = assoc_project(v[h], cam, F, T, g[h], j[h]);
    }
    float4 q[2], m[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        q[h] = ok[h] ? pv[j[h]] : zero;
        m[h] = ok[h] ? pn[j[h]] : zero;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (ok[h]) ok[h] = assoc_finish(g[h], nn[h], q[h], m[h], T, dist_th, ang_th, a[h], b[h]);
}

// The precision form's association: the gates, matched pixel, row a and residual b of
// assoc_project + assoc_finish (sensor_pose_estimation.cu:20-131), in FP32 with the
// arithmetic arranged for fewer instructions -- products fused into FMAs, the
// perspective division by one approximate reciprocal (q = p.x * rcp(p.z), |error| of a
// few ulps), round(q) as floor(q + 0.5) (the same for the q >= 0 that can pass), the
// distance gate on the squared distance, and the angle gate acos(<Rn/|Rn|, m/|m|>) <= th
// as a comparison of <Rn, m>^2 with cos^2(th) |Rn|^2 |m|^2 (with the sign of <Rn, m>)
// that needs neither normalisation nor acos.  The terms are the same functions of the
// same inputs; a pixel whose projection lies within a few ulps of a pixel boundary, or
// whose distance or angle lies within an ulp of its gate, may be decided differently
// from the plain form (a few dozen pixels of 307 200 at 640x480).
__device__ __forceinline__ bool lean_project(float4 v, const Camera& cam, const float* F, const float* T, float3& g,
                                             int& j)
{
    if (!(v.z != 0 && v.w != 0)) return false;
    const float cx = fmaf(F[0], v.x, fmaf(F[1], v.y, fmaf(F[2], v.z, F[3])));
    const float cy = fmaf(F[4], v.x, fmaf(F[5], v.y, fmaf(F[6], v.z, F[7])));
    const float cz = fmaf(F[8], v.x, fmaf(F[9], v.y, fmaf(F[10], v.z, F[11])));
    const float* K = cam.K;
    const float px = fmaf(K[0], cx, fmaf(K[1], cy, K[2] * cz));
    const float py = fmaf(K[3], cx, fmaf(K[4], cy, K[5] * cz));
    const float pz = fmaf(K[6], cx, fmaf(K[7], cy, K[8] * cz));
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(pz));
    // NaN converts to 0 and +-inf saturate: all outside the image, like the reference
    const int u = (int)floorf(fmaf(px, r, 0.5f));
    const int vv = (int)floorf(fmaf(py, r, 0.5f));
    if (!(u > 0 && u <= cam.W && vv > 0 && vv <= cam.H)) return false;
    g.x = fmaf(T[0], v.x, fmaf(T[1], v.y, fmaf(T[2], v.z, T[3])));
    g.y = fmaf(T[4], v.x, fmaf(T[5], v.y, fmaf(T[6], v.z, T[7])));
    g.z = fmaf(T[8], v.x, fmaf(T[9], v.y, fmaf(T[10], v.z, T[11])));
    j = (vv - 1) * cam.W + (u - 1);
    return true;
}

__device__ __forceinline__ bool lean_finish(float3 g, float4 n, float4 q, float4 m, const float* T, float dist2,
                                            float cos_th, float (&a)[6], float& b)
{
    const float dx = g.x - q.x, dy = g.y - q.y, dz = g.z - q.z;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (!(d2 <= dist2)) return false;
    const float rx = fmaf(T[0], n.x, fmaf(T[1], n.y, T[2] * n.z));
    const float ry = fmaf(T[4], n.x, fmaf(T[5], n.y, T[6] * n.z));
    const float rz = fmaf(T[8], n.x, fmaf(T[9], n.y, T[10] * n.z));
    const float ct = fmaf(rx, m.x, fmaf(ry, m.y, rz * m.z));
    const float nn = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float mm = fmaf(m.x, m.x, fmaf(m.y, m.y, m.z * m.z));
    const float lhs = ct * ct, rhs = (cos_th * cos_th) * (nn * mm);
    // a zero normal is NaN in the reference and rejects; so does NaN here
    const bool ang = cos_th >= 0.f ? (ct > 0.f && lhs >= rhs) : (ct >= 0.f || lhs <= rhs);
    if (!(nn > 0.f && mm > 0.f && ang)) return false;
    a[0] = fmaf(g.z, m.y, -(g.y * m.z));
    a[1] = fmaf(g.x, m.z, -(g.z * m.x));
    a[2] = fmaf(g.y, m.x, -(g.x * m.y));
    a[3] = m.x;
    a[4] = m.y;
    a[5] = m.z;
    b = -fmaf(m.x, dx, fmaf(m.y, dy, m.z * dz));  // m . (q - g)
    return true;
}

// associate_pair_from with the precision form's arithmetic: both projections, then both
// gathers, then both gates
__device__ __forceinline__ void lean_pair(const float4 (&v)[2], const float4 (&nn)[2], const float4* __restrict__ pv,
                                          const float4* __restrict__ pn, const Camera& cam, const float* F,
                                          const float* T, float dist2, float cos_th, bool (&ok)[2], float (&a)[2][6],
                                          float (&b)[2], int (&j)[2])
{
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 g[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        j[h] = -1;
        ok[h] = lean_project(v[h], cam, F, T, g[h], j[h]);
    }
    float4 q[2], m[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        q[h] = ok[h] ? pv[j[h]] : zero;
        m[h] = ok[h] ? pn[j[h]] : zero;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (ok[h]) ok[h] = lean_finish(g[h], nn[h], q[h], m[h], T, dist2, cos_th, a[h], b[h]);
}

// Deterministic block reduction: butterfly shuffles within each warp, then warp
// partials summed in warp order by threads 0..kIcpVals-1.  Result in out[] (shared).
template <bool PRECISE>
__device__ __forceinline__ void block_reduce(Acc<PRECISE>& acc, float* sh_hi, float* sh_lo, float* out_hi,
                                             float* out_lo)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int nw = kIcpBlock / 32;
#pragma unroll
    for (int k = 0; k < kIcpVals; ++k) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float h = __shfl_xor_sync(0xffffffffu, acc.hi[k], off);
            const float l = PRECISE ? __shfl_xor_sync(0xffffffffu, acc.lo[PRECISE ? k : 0], off) : 0.f;
            acc.add_pair(k, h, l);
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kIcpVals; ++k) {
            sh_hi[warp * kIcpVals + k] = acc.hi[k];
            if (PRECISE) sh_lo[warp * kIcpVals + k] = acc.lo[PRECISE ? k : 0];
        }
    }
    __syncthreads();
    if (threadIdx.x < kIcpVals) {
        const int k = threadIdx.x;
        float h = sh_hi[k], l = PRECISE ? sh_lo[k] : 0.f;
        for (int w = 1; w < nw; ++w) {
            if (PRECISE) {
                float s, e;
                two_sum(h, sh_hi[w * kIcpVals + k], s, e);
                h = s;
                l += e + sh_lo[w * kIcpVals + k];
            } else {
                h += sh_hi[w * kIcpVals + k];
            }
        }
        out_hi[k] = h;
        if (PRECISE) out_lo[k] = l;
    }
    __syncthreads();
}

__device__ __forceinline__ int tri(int r, int s) { return 6 + r * 6 - r * (r - 1) / 2 + (s - r); }

// Solve the 6x6 system from the reduced sums, apply the small-angle increment to the
// pose and prepare the next iteration (sensor_pose_estimation.cu:389-429), bit for bit
// as cv::Cholesky and cv::Mat's product do it, by the 32 lanes of one warp (warp_chol6
// and mat4_entry: FP64 latency dominates this step on GB300, so the double sums are
// carried in float pairs).  All 32 lanes of the calling warp must call.
// T0 and Tprev_inv: the state's T and Tprev_inv, already loaded by the caller (shared
// memory), so their global-memory latency overlaps the reduction; it: the state's iter
__device__ void finish_iteration_warp(State* st, const IcpParams& prm, const float* sums, const float* T0,
                                      const float* Tprev_inv, int it)
{
    __shared__ float L[36], xb[6], inc[16], Tn[16];
    __shared__ int fail;
    const int lane = threadIdx.x & 31;
    if (lane < 6) {
        xb[lane] = sums[lane];
        for (int c = 0; c <= lane; ++c) L[lane * 6 + c] = sums[tri(c, lane)];  // lower triangle of A
    }
    __syncwarp();
    const bool ok = warp_chol6(L, xb, &fail);
    if (lane == 0) {
        if (!ok && prm.fail_mode == 1)
            for (int i = 0; i < 6; ++i) xb[i] = 0.f;
        increment(xb, inc);
    }
    __syncwarp();
    // T <- Inc * T and F <- T_prev^-1 * T, one output entry per lane
    if (lane < 16) Tn[lane] = mat4_entry(inc, T0, lane);
    __syncwarp();
    if (lane < 16) {
        st->T[lane] = Tn[lane];
        st->F[lane] = mat4_entry(Tprev_inv, Tn, lane);
    }
    if (it < kMaxIcpIters && lane < 16) st->Tlog[it][lane] = Tn[lane];
    if (lane < kIcpVals) st->sums[lane] = sums[lane];
    __syncwarp();
    if (lane == 0) {
        if (it < kMaxIcpIters) {
            st->ncorr[it] = (int32_t)sums[kIcpVals - 1];
            st->chol_ok[it] = ok ? 1 : 0;
        }
        st->iter = it + 1;
    }
}

// The precision form's update by the first two warps of the last block (threads 0..63
// call; S: the sums as FP64 in shared memory, sum k: b, then A's upper triangle by rows,
// then the correspondence count): the FP64 solve (pair_gj6_f64 on named barriers 1 and
// 2), and the SE(3) composition Inc * T applied to the FP64 pose by the first warp (the
// only FP64 steps); the float pose and F follow from it.  The previous pose is loaded
// first so that its latency hides behind the solve.
__device__ void finish_precise_pair(State* st, const IcpParams& prm, const double* S)
{
    __shared__ double gj_buf[2][6][8], gj_x[6];
    __shared__ float Tf[16], Tp[16];
    const int t = threadIdx.x, lane = t & 31;
    const float tp = t < 16 ? st->Tprev_inv[t] : 0.f;
    const double td = t < 16 ? st->Td[t] : 0.0;
    const int it = st->iter;
    const auto entry = [S](int r, int c) { return c == 6 ? S[r] : S[tri(min(r, c), max(r, c))]; };
    const bool ok = pair_gj6_f64(entry, t, gj_buf, gj_x, 1);
    if (t >= 32) return;
    // the increment (omega, t) in every lane; where A is not positive definite the
    // reference applies b as it stands, or the identity in that fail mode
    double x[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) x[i] = ok ? gj_x[i] : (prm.fail_mode == 1 ? 0.0 : S[i]);
    // row rr of Inc = [[1, w2, -w1, t0], [-w2, 1, w0, t1], [w1, -w0, 1, t2], [0, 0, 0, 1]]
    const int rr = (lane >> 2) & 3, c = lane & 3;
    const double i0 = rr == 0 ? 1.0 : rr == 1 ? -x[2] : rr == 2 ? x[1] : 0.0;
    const double i1 = rr == 0 ? x[2] : rr == 1 ? 1.0 : rr == 2 ? -x[0] : 0.0;
    const double i2 = rr == 0 ? -x[1] : rr == 1 ? x[0] : rr == 2 ? 1.0 : 0.0;
    const double i3 = rr == 0 ? x[3] : rr == 1 ? x[4] : rr == 2 ? x[5] : 1.0;
    const double t0 = __shfl_sync(0xffffffffu, td, c), t1 = __shfl_sync(0xffffffffu, td, 4 + c);
    const double t2 = __shfl_sync(0xffffffffu, td, 8 + c), t3 = __shfl_sync(0xffffffffu, td, 12 + c);
    double tn = i0 * t0;
    tn = fma(i1, t1, tn);
    tn = fma(i2, t2, tn);
    tn = fma(i3, t3, tn);
    if (lane < 16) {
        st->Td[lane] = tn;
        Tf[lane] = (float)tn;
        Tp[lane] = tp;
        st->T[lane] = (float)tn;
    }
    __syncwarp();
    if (lane < 16) {
        const float f = mat4_entry(Tp, Tf, lane);
        st->F[lane] = f;
        if (it < kMaxIcpIters) st->Tlog[it][lane] = Tf[lane];
    }
    // the statistics after the pose (their conversions would queue on the FP64 pipe
    // ahead of the composition)
    if (lane < kIcpVals) st->sums[lane] = (float)S[lane];
    if (lane == 0) {
        if (it < kMaxIcpIters) {
            st->ncorr[it] = (int32_t)S[kIcpVals - 1];
            st->chol_ok[it] = ok ? 1 : 0;
        }
        st->iter = it + 1;
    }
}

// MODE 0: one ICP iteration (F, T from the state; the last block updates the pose).
// MODE 1: association + reduction at the given F, T; the last block writes the sums.
template <int MODE>
__global__ void __launch_bounds__(kIcpBlock) icp_kernel(const float4* __restrict__ vmap, const float4* __restrict__ nmap,
                                                      const float4* __restrict__ pv, const float4* __restrict__ pn,
                                                      Camera cam, IcpParams prm, State* st, const float* Fsrc,
                                                      const float* Tsrc, float* partials, float* sums_out,
                                                      int32_t* pair)
{
    __shared__ float sF[16], sT[16];
    __shared__ float sh_hi[(kIcpBlock / 32) * kIcpVals];
    __shared__ float sh_lo[1];
    __shared__ float red_hi[kIcpVals], red_lo[kIcpVals];
    __shared__ int is_last;
    if (threadIdx.x < 16) {
        sF[threadIdx.x] = Fsrc[threadIdx.x];
        sT[threadIdx.x] = Tsrc[threadIdx.x];
    }
    __syncthreads();

    Acc<false> acc;
    acc.zero();
    const int n = cam.H * cam.W;
    for (int i = blockIdx.x * kIcpBlock + threadIdx.x; i < n; i += gridDim.x * kIcpBlock) {
        float a[6], b;
        int j = -1;
        const bool ok = associate(i, vmap, nmap, pv, pn, cam, sF, sT, prm.dist, prm.angle_deg, a, b, j);
        if (MODE == 1 && pair) pair[i] = ok ? j : -1;
        if (!ok) continue;
#pragma unroll
        for (int r = 0; r < 6; ++r) acc.add(r, a[r] * b);
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
            for (int s = r; s < 6; ++s) acc.add(tri(r, s), a[r] * a[s]);
        acc.add(kIcpVals - 1, 1.f);
    }
    block_reduce<false>(acc, sh_hi, sh_lo, red_hi, red_lo);

    // publish this block's partial; the last block to arrive finishes the reduction
    float* part_hi = partials;
    if (threadIdx.x < kIcpVals) {
        part_hi[blockIdx.x * kIcpVals + threadIdx.x] = red_hi[threadIdx.x];
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(&st->ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();

    acc.zero();
    for (int bidx = threadIdx.x; bidx < (int)gridDim.x; bidx += kIcpBlock) {
#pragma unroll
        for (int k = 0; k < kIcpVals; ++k)
            acc.add_pair(k, __ldcg(part_hi + bidx * kIcpVals + k), 0.f);
    }
    block_reduce<false>(acc, sh_hi, sh_lo, red_hi, red_lo);
    if (threadIdx.x >= 32) return;
    if (threadIdx.x == 0) st->ticket = 0u;
    if (MODE == 1) {
        if (threadIdx.x < kIcpVals) sums_out[threadIdx.x] = red_hi[threadIdx.x];
        return;
    }
    __shared__ float sT0[16], sTp[16];
    if (threadIdx.x < 16) {
        sT0[threadIdx.x] = st->T[threadIdx.x];
        sTp[threadIdx.x] = st->Tprev_inv[threadIdx.x];
    }
    __syncwarp();
    finish_iteration_warp(st, prm, red_hi, sT0, sTp, st->iter);
}

// ---- reference summation order ----------------------------------------------------
// Sum_Array (sensor_pose_estimation.cu:225-245) reduces each plane in blocks of 64
// consecutive pixels with the tree sdata[t] += sdata[t + s], s = 32, 16, ..., 1, and the
// host then adds the 4800 block sums one after another in block order (:369-372).  Here
// one warp owns a 64-pixel group: lane t holds pixel t and adds pixel t + 32 (the s = 32
// step), then shuffles down by 16, 8, 4, 2, 1 -- the same additions on the same operands,
// so each group sum is bit-identical to the reference's.  The reduce pass then adds the
// group sums in group order.  Groups without a correspondence sum to +0 in every term,
// and adding +0 to a running sum that starts at +0 never changes it, so those groups are
// skipped without changing a bit.  Two launches: a group pass over all SMs and a
// one-CTA reduce-and-solve pass.
constexpr int kExactWarps = 8;

__device__ __forceinline__ void add_terms(float (&v)[kIcpVals], const float (&a)[6], float b)
{
#pragma unroll
    for (int r = 0; r < 6; ++r) v[r] = v[r] + a[r] * b;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int s = r; s < 6; ++s) v[tri(r, s)] = v[tri(r, s)] + a[r] * a[s];
    v[kIcpVals - 1] = v[kIcpVals - 1] + 1.f;
}

// add_terms with each product fused into its addition (the precision form)
__device__ __forceinline__ void add_terms_fused(float (&v)[kIcpVals], const float (&a)[6], float b)
{
#pragma unroll
    for (int r = 0; r < 6; ++r) v[r] = fmaf(a[r], b, v[r]);
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int s = r; s < 6; ++s) v[tri(r, s)] = fmaf(a[r], a[s], v[tri(r, s)]);
    v[kIcpVals - 1] = v[kIcpVals - 1] + 1.f;
}

// Group pass: one warp per 64-pixel group writes the group's 28 sums (27 terms and
// the correspondence count) and whether the group has a correspondence.
// The group sums (plain form) are stored quad-interleaved: for each quad of four
// consecutive groups, term k's four values are adjacent (float4 k of the quad), so the
// in-order reduction reads four groups of a term with one 16-byte load.
constexpr int kQuad = 4;
constexpr int kQuadFloats = kQuad * kIcpVals;  // 112 floats = 448 bytes per quad
__device__ __forceinline__ size_t partial_index(int grp, int term)
{
    return (size_t)(grp >> 2) * kQuadFloats + term * kQuad + (grp & 3);
}

// Sums each of the 28 values over the warp; lane l < 28 returns the sum of value l.  A
// butterfly in which every exchange halves the values a lane carries: 16 + 8 + 4 + 2 + 1
// shuffles in all, where a sum per value and level takes 28 per level.  At the exchange
// of width w a lane adds, for each value it keeps, its own partial at position p and its
// partner's at p ^ w, so every value is summed by the pairs (t, t + w), w = 16, 8, 4, 2,
// 1 -- the reference's shared-memory tree (sensor_pose_estimation.cu:225-245) after its
// stride-32 step, with each addition's operands in either order (addition commutes).
__device__ __forceinline__ float warp_sum_transposed(const float (&v)[kIcpVals])
{
    const int lane = threadIdx.x & 31;
    float a[16];
    {
        const bool up = lane & 16;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const float lo = v[k], hi = k + 16 < kIcpVals ? v[k + 16] : 0.f;
            a[k] = (up ? hi : lo) + __shfl_xor_sync(0xffffffffu, up ? lo : hi, 16);
        }
    }
#pragma unroll
    for (int w = 8; w >= 1; w >>= 1) {
        const bool up = lane & w;
#pragma unroll
        for (int k = 0; k < w; ++k) {
            const float lo = a[k], hi = a[k + w];
            a[k] = (up ? hi : lo) + __shfl_xor_sync(0xffffffffu, up ? lo : hi, w);
        }
    }
    return a[0];
}

// group_sums with the lane's two vertices and normals already loaded (load_pair)
template <int MODE>
__device__ __forceinline__ void group_sums_from(int grp, int lane, const float4 (&vx)[2], const float4 (&nx)[2],
                                                const float4* __restrict__ pv, const float4* __restrict__ pn,
                                                const Camera& cam, const IcpParams& prm, const float* sF,
                                                const float* sT, float* __restrict__ partials,
                                                int* __restrict__ flags, int32_t* __restrict__ pair)
{
    const int n = cam.H * cam.W;
    float v[kIcpVals];
#pragma unroll
    for (int k = 0; k < kIcpVals; ++k) v[k] = 0.f;
    bool ok[2];
    float a[2][6], b[2];
    int j[2];
    associate_pair_from(vx, nx, pv, pn, cam, sF, sT, prm.dist, prm.angle_deg, ok, a, b, j);
    if (MODE == 1 && pair) {
        if (grp * 64 + lane < n) pair[grp * 64 + lane] = ok[0] ? j[0] : -1;
        if (grp * 64 + 32 + lane < n) pair[grp * 64 + 32 + lane] = ok[1] ? j[1] : -1;
    }
    if (ok[0]) add_terms(v, a[0], b[0]);  // v = terms of pixel t (0 + x == x up to the sign of a zero)
    if (ok[1]) {
        float w[kIcpVals];
#pragma unroll
        for (int k = 0; k < kIcpVals; ++k) w[k] = 0.f;
        add_terms(w, a[1], b[1]);
#pragma unroll
        for (int k = 0; k < kIcpVals; ++k) v[k] = v[k] + w[k];  // sdata[t] += sdata[t + 32]
    }
    // the rest of the tree, strides 16 .. 1, for all 28 values at once; lane k keeps value k
    const float vs = warp_sum_transposed(v);
    if (lane < kIcpVals) partials[partial_index(grp, lane)] = vs;
    if (lane == kIcpVals - 1) flags[grp] = vs != 0.f ? 1 : 0;
}

template <int MODE>
__device__ __forceinline__ void group_sums(int grp, int lane, const float4* __restrict__ vmap,
                                           const float4* __restrict__ nmap, const float4* __restrict__ pv,
                                           const float4* __restrict__ pn, const Camera& cam, const IcpParams& prm,
                                           const float* sF, const float* sT, float* __restrict__ partials,
                                           int* __restrict__ flags, int32_t* __restrict__ pair)
{
    float4 vx[2], nx[2];
    load_pair(grp * 64 + lane, cam.H * cam.W, vmap, nmap, vx, nx);
    group_sums_from<MODE>(grp, lane, vx, nx, pv, pn, cam, prm, sF, sT, partials, flags, pair);
}

template <int MODE>
__global__ void __launch_bounds__(kExactWarps * 32, 4) icp_group_kernel(
    const float4* __restrict__ vmap, const float4* __restrict__ nmap, const float4* __restrict__ pv,
    const float4* __restrict__ pn, Camera cam, IcpParams prm, const float* Fsrc, const float* Tsrc,
    float* __restrict__ partials, int* __restrict__ flags, int ngroups, int32_t* __restrict__ pair, int prefetch)
{
    // one group per warp (the grid covers the groups)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = blockIdx.x * kExactWarps + warp;
    const int n = cam.H * cam.W;
    // The vertex and normal maps are written before the frame's first ICP pass and never
    // by a pass, so after a pass (prefetch) they are loaded before waiting for it: the
    // first round of loads overlaps the previous pass's reduction and solve.
    float4 vx[2], nx[2];
    if (prefetch) load_pair(grp * 64 + lane, n, vmap, nmap, vx, nx);
    wait_for_producer();
    // the solve pass may be scheduled now: it waits for this pass before reading its sums
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (!prefetch) load_pair(grp * 64 + lane, n, vmap, nmap, vx, nx);
    __shared__ float sF[16], sT[16];
    if (threadIdx.x < 16) {
        sF[threadIdx.x] = Fsrc[threadIdx.x];
        sT[threadIdx.x] = Tsrc[threadIdx.x];
    }
    __syncthreads();
    if (grp < ngroups) group_sums_from<MODE>(grp, lane, vx, nx, pv, pn, cam, prm, sF, sT, partials, flags, pair);
}

// the group pass of every scene of a batch at pyramid level `level`; WARPS warps per
// block (a shape the batch's autotuner picks)
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) icp_group_batch_kernel(const SceneDev* __restrict__ scenes, int level)
{
    wait_for_producer();
    const SceneDev& d = scenes[blockIdx.y];
    const Camera& cam = d.cam[level];
    const int ngroups = (cam.H * cam.W + 63) / 64;
    if ((int)blockIdx.x * WARPS >= ngroups) return;
    __shared__ float sF[16], sT[16];
    if (threadIdx.x < 16) {
        sF[threadIdx.x] = d.st->F[threadIdx.x];
        sT[threadIdx.x] = d.st->T[threadIdx.x];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = blockIdx.x * WARPS + warp;
    if (grp < ngroups)
        group_sums<0>(grp, lane, d.vmap[level], d.nmap[level], d.pv[level], d.pn[level], cam, d.icp, sF, sT,
                      d.partials, d.groups, nullptr);
}

// the group pass of every scene of a batch at `level`, spread over a fixed grid: warp w
// of the grid takes the groups w, w + W, w + 2W, ... of the flattened list of all scenes'
// groups (scene s owns groups [grp_start of s, grp_start of s + 1)); groups cost about
// the same, so a static share needs no counter
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) icp_group_batch_persist_kernel(const SceneDev* __restrict__ scenes,
                                                                           int n_scenes, int level, unsigned total)
{
    wait_for_producer();
    __shared__ float sF[WARPS][16], sT[WARPS][16];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int cur = -1;
    for (unsigned g = blockIdx.x * WARPS + warp; g < total; g += gridDim.x * WARPS) {
        int s = 0;
        while (s + 1 < n_scenes && g >= (unsigned)scenes[s + 1].grp_start[level]) ++s;
        const SceneDev& d = scenes[s];
        if (s != cur) {
            __syncwarp();
            if (lane < 16) {
                sF[warp][lane] = d.st->F[lane];
                sT[warp][lane] = d.st->T[lane];
            }
            __syncwarp();
            cur = s;
        }
        group_sums<0>((int)(g - (unsigned)d.grp_start[level]), lane, d.vmap[level], d.nmap[level], d.pv[level],
                      d.pn[level], d.cam[level], d.icp, sF[warp], sT[warp], d.partials, d.groups, nullptr);
    }
}

// Reduce-and-solve pass: one warp.  The group sums are streamed into shared memory in
// order by the bulk-copy engine (cp.async.bulk into a ring of kBuffers chunks with
// mbarrier completion; kBuffers - 1 copies stay in flight) while the warp adds them:
// lane k keeps the running sum of term k.  The additions run as one software pipeline
// over batches of kBatchQ quads (16 groups) -- the next batch's shared-memory loads are
// issued before the current batch's additions, across chunk boundaries too -- so the
// serial part is the FADD chain itself; a lane reads a quad's four values of its term
// with one 16-byte load and adds them in group order.  Empty groups sum to +0 and are
// added like the rest (exact).  Then the warp solves and updates the pose (MODE 0) or
// writes the sums (MODE 1).
constexpr int kChunkGroups = 512;                               // 512 x 112 B = 56 KB
constexpr int kBuffers = 3;  // 3 x 56 KB: two copies in flight (the third buffer saved 3.7 us per c1 frame)
constexpr int kBatchQ = 4;                                      // quads per batch
constexpr int kBatchesPerChunk = kChunkGroups / (kQuad * kBatchQ);
static_assert(kChunkGroups % (2 * kQuad * kBatchQ) == 0, "a chunk is an even number of batches");
constexpr unsigned kChunkBytes = kChunkGroups * kIcpVals * 4u;  // multiple of 16

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// bounded wait for the phase of the given parity: false once `limit` polls have passed
// without it (State::wait_limit; a copy that has not landed by then is reported, not
// awaited)
__device__ __forceinline__ bool bar_wait(unsigned long long* bar, unsigned parity, long long limit)
{
    for (long long i = 0; i < limit; ++i) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int MODE>
__device__ __forceinline__ void solve_body(const float* __restrict__ partials, int ngroups, State* st,
                                           const IcpParams& prm, float* sums_out)
{
    extern __shared__ float4 smem4[];
    float* buf = reinterpret_cast<float*>(smem4);  // kBuffers x kChunkGroups x kIcpVals
    __shared__ __align__(8) unsigned long long bars[kBuffers];
    __shared__ float red[kIcpVals];
    __shared__ float sT0[16], sTp[16];
    const int lane = threadIdx.x;
    const long long limit = st->wait_limit;
    // the pose inputs of the solve, loaded now so their latency hides behind the sums
    float t0 = 0.f, tp = 0.f;
    int it = 0;
    if (MODE == 0) {
        if (lane < 16) {
            t0 = st->T[lane];
            tp = st->Tprev_inv[lane];
        }
        it = st->iter;
    }
    const int nchunks = (ngroups + kChunkGroups - 1) / kChunkGroups;
    // whole quads: a partial last quad is copied whole (the buffer holds whole quads; the
    // values past ngroups are not added)
    auto chunk_bytes = [&](int c) {
        return (unsigned)((min(kChunkGroups, ngroups - c * kChunkGroups) + kQuad - 1) / kQuad * kQuadFloats * 4);
    };
    if (lane == 0) {
        for (int k = 0; k < kBuffers; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[k])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int c = 0; c < kBuffers && c < nchunks; ++c)
            bulk_load(buf + c * kChunkGroups * kIcpVals, partials + (size_t)c * kChunkGroups * kIcpVals,
                      chunk_bytes(c), &bars[c]);
    }
    __syncwarp();
    // chunks issued so far (uniform over the warp), and the chunk whose wait gave up
    int issued = min(kBuffers, nchunks), failed_at = 0;
    // lanes 28..31 read term 27's values too (in bounds) and discard them
    const int term = lane < kIcpVals ? lane : kIcpVals - 1;
    // quad q of chunk c's slot, this lane's term: float4 q * kIcpVals + term
    auto slot_ptr = [&](int c) {
        return reinterpret_cast<const float4*>(buf + (c % kBuffers) * kChunkGroups * kIcpVals) + term;
    };
    float sum = 0.f;
    auto add4 = [&](const float4& q) {
        sum = sum + q.x;
        sum = sum + q.y;
        sum = sum + q.z;
        sum = sum + q.w;
    };
    bool ok = nchunks == 0 || bar_wait(&bars[0], 0, limit);
    const int full = ngroups / kChunkGroups;  // chunks of exactly kChunkGroups groups
    float4 va[kBatchQ], vb[kBatchQ];
    if (ok && full > 0) {
        const float4* p = slot_ptr(0);
#pragma unroll
        for (int q = 0; q < kBatchQ; ++q) va[q] = p[q * kIcpVals];
    }
    for (int c = 0; c < full && ok; ++c) {
        // batches 0..kBatchesPerChunk-1 of chunk c; va holds batch 0 on entry.  The next
        // batch's loads are issued before the current batch's additions.
        const float4* p = slot_ptr(c);
        for (int i = 0; i < kBatchesPerChunk - 2; i += 2) {
#pragma unroll
            for (int q = 0; q < kBatchQ; ++q) {
                vb[q] = p[((i + 1) * kBatchQ + q) * kIcpVals];
                add4(va[q]);
            }
#pragma unroll
            for (int q = 0; q < kBatchQ; ++q) {
                va[q] = p[((i + 2) * kBatchQ + q) * kIcpVals];
                add4(vb[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < kBatchQ; ++q) {
            vb[q] = p[((kBatchesPerChunk - 1) * kBatchQ + q) * kIcpVals];
            add4(va[q]);
        }
        // open the next full chunk before the last batch's additions
        if (c + 1 < full) {
            ok = bar_wait(&bars[(c + 1) % kBuffers], ((c + 1) / kBuffers) & 1, limit);
            if (!ok) failed_at = c + 1;
            const float4* pn = slot_ptr(c + 1);
#pragma unroll
            for (int q = 0; q < kBatchQ; ++q) va[q] = ok ? pn[q * kIcpVals] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < kBatchQ; ++q) add4(vb[q]);
        // every group of chunk c is added: its slot goes back to the copy engine
        __syncwarp();
        if (ok && c + kBuffers < nchunks) {
            if (lane == 0) {
                // the warp's reads of this slot precede the async-proxy write that refills it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                bulk_load(buf + (c % kBuffers) * kChunkGroups * kIcpVals,
                          partials + (size_t)(c + kBuffers) * kChunkGroups * kIcpVals, chunk_bytes(c + kBuffers),
                          &bars[c % kBuffers]);
            }
            issued = c + kBuffers + 1;
        }
    }
    if (ok && full < nchunks) {
        // the last, partial chunk: whole quads, then the groups of a partial last quad
        if (full > 0) {
            ok = bar_wait(&bars[full % kBuffers], (full / kBuffers) & 1, limit);
            if (!ok) failed_at = full;
        }
        if (ok) {
            const float4* p = slot_ptr(full);
            const int cnt = ngroups - full * kChunkGroups;
            const int nq = cnt / kQuad, rem = cnt % kQuad;
            int r = 0;
            for (; r + kBatchQ <= nq; r += kBatchQ) {
#pragma unroll
                for (int q = 0; q < kBatchQ; ++q) va[q] = p[(r + q) * kIcpVals];
#pragma unroll
                for (int q = 0; q < kBatchQ; ++q) add4(va[q]);
            }
            for (; r < nq; ++r) add4(p[r * kIcpVals]);
            if (rem) {
                const float4 t = p[nq * kIcpVals];
                sum = sum + t.x;
                if (rem > 1) sum = sum + t.y;
                if (rem > 2) sum = sum + t.z;
            }
        }
    }
    if (!ok) {
        // A bulk copy did not complete within the limit: report it, and leave the pose as
        // it is (MODE 1 writes NaN sums, so a failed reduction cannot pass for a result).
        // The copies still in flight -- chunks failed_at .. issued-1, each the only one
        // outstanding on its buffer -- get a bounded wait at the default limit before the
        // block exits, so none lands in shared memory the block no longer owns.
        if (lane == 0) st->error = 1;
        if (MODE == 1 && lane < kIcpVals) sums_out[lane] = qnan();
        if (lane == 0)
            for (int c = failed_at; c < issued; ++c)
                bar_wait(&bars[c % kBuffers], (c / kBuffers) & 1, kDefaultWaitLimit);
        return;
    }
    if (lane < kIcpVals) red[lane] = sum;
    __syncwarp();
    if (MODE == 1) {
        if (lane < kIcpVals) sums_out[lane] = red[lane];
        return;
    }
    if (lane < 16) {
        sT0[lane] = t0;
        sTp[lane] = tp;
    }
    __syncwarp();
    finish_iteration_warp(st, prm, red, sT0, sTp, it);
}

// The precision form in one pass per iteration.  One warp per 64-pixel group forms the
// group's 28 sums (as in the group pass); the block combines its groups with
// compensated (TwoSum) FP32 into a hi/lo pair per sum, and adds both to an exact
// fixed-point accumulator: each value times 2^48, truncated toward zero, as a 128-bit
// two's-complement integer whose four 32-bit digits go to four 64-bit accumulators by
// atomic addition (integer addition commutes, so the result does not depend on the
// order the blocks arrive in).  The last block to finish (a ticket) reads and clears
// the accumulators, carries the digits into one integer per sum, converts it to FP64
// and solves (finish_precise_pair, MODE 0) or writes the float sums (MODE 1).  Nothing
// waits for a second pass over the partials.  Every block value below 2^79 in magnitude
// is held exactly (to 2^-48), and the digit accumulators stay below 2^63 for fewer than
// 2^31 blocks, so their sum is exact; a non-finite or larger block value marks its sum
// NaN, as the float sum would have gone infinite or NaN.  The accumulators are spread
// over kFixReplicas copies (block b adds to copy b % kFixReplicas), so that few atomic
// additions queue on any one word; within a copy the 112 digits are consecutive, so a
// block's additions and the last block's reads are whole-line (coalesced) accesses.
// warps per block of the precision form's pass (32 / kPreciseWarps blocks per SM at
// 64 registers a thread)
constexpr int kPreciseWarps = 8;

namespace fix {

// f * 2^48 truncated toward zero as a 128-bit two's-complement integer (hi, lo); false
// for a non-finite f or |f| >= 2^79
__device__ __forceinline__ bool to_fixed(float f, unsigned long long& hi, unsigned long long& lo)
{
    const unsigned u = __float_as_uint(f);
    const int e = (int)((u >> 23) & 0xffu);
    hi = lo = 0ull;
    if (e == 0xff || e > 205) return false;
    const unsigned long long m = (u & 0x7fffffu) | (e ? 0x800000u : 0u);
    const int sh = (e ? e : 1) - 102;  // |f| * 2^48 = m * 2^sh, m < 2^24, sh <= 103
    if (sh >= 64) {
        hi = m << (sh - 64);
    } else if (sh > 40) {
        hi = m >> (64 - sh);
        lo = m << sh;
    } else if (sh >= 0) {
        lo = m << sh;
    } else if (sh > -64) {
        lo = m >> (-sh);
    }
    if (u >> 31) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    return true;
}

constexpr int kFixReplicas = 16;
constexpr int kDigits = kIcpVals * 4;  // words per copy: 7 lines of 128 bytes

// copy r of the accumulators: kDigits consecutive words, digit d of sum k at k * 4 + d
__device__ __forceinline__ unsigned long long* copy_of(long long* acc, int r)
{
    return reinterpret_cast<unsigned long long*>(acc) + (size_t)r * kDigits;
}

// the four digits of hi + lo (a compensated pair): three unsigned 32-bit digits and the
// signed top digit; false (digits zero) if either part cannot be represented
__device__ __forceinline__ bool digits_of(float h, float l, unsigned long long (&dg)[4])
{
    unsigned long long h1, l1, h2, l2;
    const bool ok = to_fixed(h, h1, l1) & to_fixed(l, h2, l2);
    const unsigned long long lo = l1 + l2;
    const unsigned long long hi = h1 + h2 + (lo < l1 ? 1ull : 0ull);
    dg[0] = ok ? lo & 0xffffffffull : 0ull;
    dg[1] = ok ? lo >> 32 : 0ull;
    dg[2] = ok ? hi & 0xffffffffull : 0ull;
    dg[3] = ok ? (unsigned long long)((long long)hi >> 32) : 0ull;
    return ok;
}

// The last block's read-out, all threads of the block: thread t < kDigits reads word t
// of every copy (each load instruction covers 32 consecutive words, and all are issued
// before any is used), adds them and clears them; digits[t] (shared) receives the sum,
// and *bad_out (shared) the flags of the sums that could not be accumulated (read and
// cleared in the same round of loads).
__device__ __forceinline__ void gather_digits(long long* acc, long long* digits, unsigned* bad_flags,
                                              unsigned* bad_out)
{
    static_assert(kDigits < kPreciseWarps * 32, "one thread per digit and one for the flags");
    const int t = threadIdx.x;
    if (t == kPreciseWarps * 32 - 1) {
        // every other block's atomicOr on the flags came before its ticket
        *bad_out = __ldcg(bad_flags);
        __stcg(bad_flags, 0u);
    }
    if (t < kDigits) {
        unsigned long long x[kFixReplicas];
#pragma unroll
        for (int i = 0; i < kFixReplicas; ++i) x[i] = __ldcg(copy_of(acc, i) + t);
        long long v = 0;
#pragma unroll
        for (int i = 0; i < kFixReplicas; ++i) {
            v += (long long)x[i];
            __stcg(copy_of(acc, i) + t, 0ull);
        }
        digits[t] = v;
    }
    __syncthreads();
}

// sum k from its carried digits (NaN if flagged)
__device__ __forceinline__ double take(const long long* digits, int k, bool flagged)
{
    const long long d0 = digits[k * 4 + 0], d1 = digits[k * 4 + 1];
    const long long d2 = digits[k * 4 + 2], d3 = digits[k * 4 + 3];
    if (flagged) return __longlong_as_double(0x7ff8000000000000ll);
    // carry the digits: V = t3 2^96 + L, L = w2 2^64 + w1 2^32 + w0 with 0 <= w < 2^32
    const long long M = 0xffffffffll;
    long long t = d0;
    const unsigned long long w0 = (unsigned long long)(t & M);
    t = d1 + (t >> 32);
    const unsigned long long w1 = (unsigned long long)(t & M);
    t = d2 + (t >> 32);
    unsigned long long lhi = (unsigned long long)(t & M);  // L = lhi 2^64 + llo
    unsigned long long llo = (w1 << 32) | w0;
    long long top = d3 + (t >> 32);
    const bool neg = top < 0;
    if (neg) {
        // |V| = (-top - 1) 2^96 + (2^96 - L), or -top 2^96 when L = 0
        if (lhi == 0ull && llo == 0ull) {
            top = -top;
        } else {
            top = -top - 1;
            const unsigned long long borrow = llo != 0ull ? 1ull : 0ull;
            llo = ~llo + 1ull;
            lhi = ((1ull << 32) - lhi - borrow) & 0xffffffffull;
        }
    }
    if (((unsigned long long)top >> 32) == 0ull) {
        // |V| < 2^128 (every sum of this pipeline): |V| 2^-48 rounded to the nearest
        // double by integer arithmetic on the 128-bit magnitude h 2^64 + l -- normalise,
        // keep 53 bits, round half to even -- so the conversion uses no FP64 instruction
        const unsigned long long h = ((unsigned long long)top << 32) | lhi, l = llo;
        if ((h | l) == 0ull) return 0.0;
        const int lz = h ? __clzll((long long)h) : 64 + __clzll((long long)l);
        unsigned long long nh;
        unsigned long long nl;
        if (lz >= 64) {
            nh = l << (lz - 64);
            nl = 0ull;
        } else if (lz == 0) {
            nh = h;
            nl = l;
        } else {
            nh = (h << lz) | (l >> (64 - lz));
            nl = l << lz;
        }
        unsigned long long mant = nh >> 11;  // 53 bits, the leading one at bit 52
        int e = 127 - lz;                    // the leading bit's exponent in |V|
        const bool half = ((nh >> 10) & 1ull) != 0ull;
        const bool sticky = (nh & 0x3ffull) != 0ull || nl != 0ull;
        if (half && (sticky || (mant & 1ull))) {
            ++mant;
            if (mant >> 53) {
                mant >>= 1;
                ++e;
            }
        }
        const unsigned long long bits = ((unsigned long long)(e - 48 + 1023) << 52) | (mant & 0xfffffffffffffull) |
                                        (neg ? (1ull << 63) : 0ull);
        return __longlong_as_double((long long)bits);
    }
    // beyond 2^128: non-negative terms from the top, a relative error of a few ulps
    double v = (double)top * 0x1p96;
    v += (double)lhi * 0x1p64;
    v += (double)llo;
    return (neg ? -v : v) * 0x1p-48;
}

}  // namespace fix

template <int MODE>
__global__ void __launch_bounds__(kPreciseWarps * 32, 32 / kPreciseWarps) icp_precise_kernel(
    const float4* __restrict__ vmap, const float4* __restrict__ nmap, const float4* __restrict__ pv,
    const float4* __restrict__ pn, Camera cam, IcpParams prm, const float* Fsrc, const float* Tsrc, State* st,
    long long* __restrict__ fixacc, int ngroups, int prefetch, int32_t* __restrict__ pair, float* sums_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = cam.H * cam.W;
    const int grp = blockIdx.x * kPreciseWarps + warp;
    // The vertex and normal maps are written before the frame's first ICP pass and never
    // by a pass, so after a pass (prefetch) they are loaded before waiting for it: the
    // first round of loads overlaps the previous pass's solve.
    float4 v[2], nn[2];
    if (prefetch) load_pair(grp * 64 + lane, n, vmap, nmap, v, nn);
    wait_for_producer();
    // the next pass may be scheduled now: it waits for this one to finish before it
    // reads anything this one writes (every kernel launched with launch_pdl does)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (!prefetch) load_pair(grp * 64 + lane, n, vmap, nmap, v, nn);
    __shared__ float sF[16], sT[16];
    __shared__ float wsum[kPreciseWarps][kIcpVals];
    __shared__ unsigned long long sdig[fix::kDigits];
    __shared__ int is_last;
    if (threadIdx.x < 16) {
        sF[threadIdx.x] = Fsrc[threadIdx.x];
        sT[threadIdx.x] = Tsrc[threadIdx.x];
    }
    __syncthreads();
    float vals[kIcpVals];
#pragma unroll
    for (int k = 0; k < kIcpVals; ++k) vals[k] = 0.f;
    if (grp < ngroups) {
        bool ok[2];
        float a[2][6], b[2];
        int j[2];
        lean_pair(v, nn, pv, pn, cam, sF, sT, prm.dist2, prm.cos_angle, ok, a, b, j);
        if (MODE == 1 && pair) {
            if (grp * 64 + lane < n) pair[grp * 64 + lane] = ok[0] ? j[0] : -1;
            if (grp * 64 + 32 + lane < n) pair[grp * 64 + 32 + lane] = ok[1] ? j[1] : -1;
        }
        if (ok[0]) add_terms_fused(vals, a[0], b[0]);
        if (ok[1]) add_terms_fused(vals, a[1], b[1]);
    }
    const float vs = warp_sum_transposed(vals);  // the whole warp: also where grp >= ngroups
    if (lane < kIcpVals) wsum[warp][lane] = vs;
    __syncthreads();
    if (threadIdx.x < kIcpVals) {
        const int k = threadIdx.x;
        float h = wsum[0][k], l = 0.f;
        for (int w = 1; w < kPreciseWarps; ++w) {
            float sum, e;
            two_sum(h, wsum[w][k], sum, e);
            h = sum;
            l += e;
        }
        unsigned long long dg[4];
        if (!fix::digits_of(h, l, dg)) atomicOr(&st->fix_bad, 1u << k);
#pragma unroll
        for (int d = 0; d < 4; ++d) sdig[k * 4 + d] = dg[d];
    }
    __syncthreads();
    // one atomic addition per digit, 32 consecutive words per instruction
    if (threadIdx.x < fix::kDigits) {
        atomicAdd(fix::copy_of(fixacc, blockIdx.x % fix::kFixReplicas) + threadIdx.x, sdig[threadIdx.x]);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // acquire: the last block's reads of the accumulators come after every block's
        // additions, which each block fenced before its ticket
        unsigned old;
        asm volatile("atom.acquire.gpu.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(&st->ticket) : "memory");
        is_last = old == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __shared__ long long digits[kIcpVals * 4];
    __shared__ unsigned bad;
    __shared__ double S[kIcpVals];
    fix::gather_digits(fixacc, digits, &st->fix_bad, &bad);
    if (threadIdx.x >= 64) return;
    const double val = threadIdx.x < kIcpVals ? fix::take(digits, threadIdx.x, (bad >> threadIdx.x) & 1u) : 0.0;
    if (threadIdx.x == 0) st->ticket = 0u;
    if (MODE == 1) {
        if (threadIdx.x < kIcpVals) sums_out[threadIdx.x] = (float)val;
        return;
    }
    if (threadIdx.x < kIcpVals) S[threadIdx.x] = val;
    pair_bar(1);
    finish_precise_pair(st, prm, S);
}

template <int MODE>
__global__ void __launch_bounds__(32, 1) icp_solve_kernel(const float* __restrict__ partials, int ngroups, State* st,
                                                        IcpParams prm, float* sums_out)
{
    wait_for_producer();
    // the next pass may be scheduled now and load what no pass writes; it waits for this
    // one before reading the pose
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    solve_body<MODE>(partials, ngroups, st, prm, sums_out);
}

// every scene's reduce-and-solve pass: one one-warp CTA per scene, all at once
__global__ void __launch_bounds__(32, 1) icp_solve_batch_kernel(const SceneDev* __restrict__ scenes, int level)
{
    wait_for_producer();
    const SceneDev& d = scenes[blockIdx.x];
    const Camera& cam = d.cam[level];
    solve_body<0>(d.partials, (cam.H * cam.W + 63) / 64, d.st, d.icp, nullptr);
}

size_t solve_smem_bytes(int /*ngroups*/) { return (size_t)kBuffers * kChunkBytes; }

// the reduce-and-solve warp needs more than the default 48 KB of dynamic shared memory
void ensure_solve_smem(int ngroups)
{
    static int configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    const int need = (int)solve_smem_bytes(ngroups);
    if (dev < 0 || dev >= 64 || configured[dev] >= need) return;
    cudaFuncSetAttribute(icp_solve_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, need);
    cudaFuncSetAttribute(icp_solve_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, need);
    cudaFuncSetAttribute(icp_solve_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, need);
    configured[dev] = need;
}

// device addresses of State members, computed without dereferencing on the host
const float* state_F(State* st) { return reinterpret_cast<const float*>(reinterpret_cast<char*>(st) + offsetof(State, F)); }
const float* state_T(State* st) { return reinterpret_cast<const float*>(reinterpret_cast<char*>(st) + offsetof(State, T)); }

int blocks_for(int H, int W)
{
    const int b = (H * W + kIcpBlock - 1) / kIcpBlock;
    return b < kIcpMaxBlocks ? (b < 1 ? 1 : b) : kIcpMaxBlocks;
}

}  // namespace

int icp_grid_blocks(int H, int W) { return blocks_for(H, W); }

int icp_groups(int H, int W) { return (H * W + 63) / 64; }

void icp_prepare(int H, int W) { ensure_solve_smem(icp_groups(H, W)); }

size_t icp_fixacc_words() { return (size_t)fix::kDigits * fix::kFixReplicas; }

size_t icp_scratch_floats(int H, int W)
{
    const size_t a = (size_t)2 * blocks_for(H, W) * kIcpVals;
    const size_t b = (size_t)((icp_groups(H, W) + kQuad - 1) / kQuad) * kQuadFloats;  // whole quads
    return a > b ? a : b;
}

namespace {
// the precision form's gate constants (lean_finish)
IcpParams lean_params(const IcpParams& prm)
{
    IcpParams q = prm;
    q.dist2 = prm.dist >= 0.f ? prm.dist * prm.dist : -1.f;
    q.cos_angle = prm.angle_deg < 0.f ? 2.f : (float)std::cos((double)prm.angle_deg * (3.14159265358979323846 / 180.0));
    return q;
}

int exact_blocks(int H, int W)
{
    const int g = icp_groups(H, W);
    return (g + kExactWarps - 1) / kExactWarps;
}

int precise_blocks(int H, int W)
{
    const int g = icp_groups(H, W);
    return (g + kPreciseWarps - 1) / kPreciseWarps;
}
}  // namespace

void launch_icp_iteration(const float4* vmap, const float4* nmap, const float4* pv, const float4* pn,
                          const Camera& cam, const IcpParams& prm, State* st, float* partials, int* list,
                          long long* fixacc, bool after_pass, cudaStream_t s)
{
    const int blocks = blocks_for(cam.H, cam.W);
    if (!prm.precise && prm.reference_order) {
        const int ng = icp_groups(cam.H, cam.W);
        ensure_solve_smem(ng);
        launch_pdl(icp_group_kernel<0>, dim3(exact_blocks(cam.H, cam.W)), dim3(kExactWarps * 32), 0, s, vmap, nmap, pv,
                   pn, cam, prm, state_F(st), state_T(st), partials, list, ng, (int32_t*)nullptr, after_pass ? 1 : 0);
        launch_pdl(icp_solve_kernel<0>, dim3(1), dim3(32), solve_smem_bytes(ng), s, (const float*)partials, ng, st,
                   prm, (float*)nullptr);
    } else if (prm.precise) {
        const int ng = icp_groups(cam.H, cam.W);
        launch_pdl(icp_precise_kernel<0>, dim3(precise_blocks(cam.H, cam.W)), dim3(kPreciseWarps * 32), 0, s, vmap, nmap,
                   pv, pn, cam, lean_params(prm), state_F(st), state_T(st), st, fixacc, ng, after_pass ? 1 : 0,
                   (int32_t*)nullptr, (float*)nullptr);
    } else
        icp_kernel<0><<<blocks, kIcpBlock, 0, s>>>(vmap, nmap, pv, pn, cam, prm, st, state_F(st), state_T(st),
                                                   partials, nullptr, nullptr);
}

void launch_icp_associate(const float4* vmap, const float4* nmap, const float4* pv, const float4* pn,
                          const Camera& cam, const IcpParams& prm, const float* F, const float* T, State* st,
                          float* partials, int* list, long long* fixacc, float* sums_out, int32_t* pair,
                          cudaStream_t s)
{
    const int blocks = blocks_for(cam.H, cam.W);
    if (!prm.precise && prm.reference_order) {
        const int ng = icp_groups(cam.H, cam.W);
        ensure_solve_smem(ng);
        launch_pdl(icp_group_kernel<1>, dim3(exact_blocks(cam.H, cam.W)), dim3(kExactWarps * 32), 0, s, vmap, nmap, pv,
                   pn, cam, prm, F, T, partials, list, ng, pair, 0);
        launch_pdl(icp_solve_kernel<1>, dim3(1), dim3(32), solve_smem_bytes(ng), s, (const float*)partials, ng, st,
                   prm, sums_out);
    } else if (prm.precise) {
        const int ng = icp_groups(cam.H, cam.W);
        launch_pdl(icp_precise_kernel<1>, dim3(precise_blocks(cam.H, cam.W)), dim3(kPreciseWarps * 32), 0, s, vmap, nmap,
                   pv, pn, cam, lean_params(prm), F, T, st, fixacc, ng, 0, pair, sums_out);
    } else
        icp_kernel<1><<<blocks, kIcpBlock, 0, s>>>(vmap, nmap, pv, pn, cam, prm, st, F, T, partials,
                                                          sums_out, pair);
}

void launch_icp_iteration_batch(const SceneDev* scenes, int n_scenes, int max_groups, int level, int warps,
                                cudaStream_t s)
{
    ensure_solve_smem(max_groups);
    switch (warps) {
    case 4:
        launch_pdl(icp_group_batch_kernel<4>, dim3((max_groups + 3) / 4, n_scenes), dim3(4 * 32), 0, s, scenes, level);
        break;
    case 16:
        launch_pdl(icp_group_batch_kernel<16>, dim3((max_groups + 15) / 16, n_scenes), dim3(16 * 32), 0, s, scenes,
                   level);
        break;
    default:
        launch_pdl(icp_group_batch_kernel<8>, dim3((max_groups + 7) / 8, n_scenes), dim3(8 * 32), 0, s, scenes, level);
    }
    launch_pdl(icp_solve_batch_kernel, dim3(n_scenes), dim3(32), solve_smem_bytes(max_groups), s, scenes, level);
}

void launch_icp_iteration_batch_persistent(const SceneDev* scenes, int n_scenes, int max_groups, int level,
                                           unsigned total_groups, int blocks, cudaStream_t s)
{
    ensure_solve_smem(max_groups);
    launch_pdl(icp_group_batch_persist_kernel<8>, dim3(blocks), dim3(8 * 32), 0, s, scenes, n_scenes, level,
               total_groups);
    launch_pdl(icp_solve_batch_kernel, dim3(n_scenes), dim3(32), solve_smem_bytes(max_groups), s, scenes, level);
}

void launch_icp_group_batch(const SceneDev* scenes, int n_scenes, int max_groups, int level, int warps, cudaStream_t s)
{
    switch (warps) {
    case 4:
        launch_pdl(icp_group_batch_kernel<4>, dim3((max_groups + 3) / 4, n_scenes), dim3(4 * 32), 0, s, scenes, level);
        break;
    case 16:
        launch_pdl(icp_group_batch_kernel<16>, dim3((max_groups + 15) / 16, n_scenes), dim3(16 * 32), 0, s, scenes,
                   level);
        break;
    default:
        launch_pdl(icp_group_batch_kernel<8>, dim3((max_groups + 7) / 8, n_scenes), dim3(8 * 32), 0, s, scenes, level);
    }
}

}  // namespace kf
