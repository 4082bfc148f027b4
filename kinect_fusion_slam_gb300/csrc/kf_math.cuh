// Small-matrix routines shared by host and device code of the kinfu_gb300 library.
//
// The reference calls OpenCV for these on the host (cv::Mat::inv at
// projective_tsdf.cu:148-149, voxel_traversal.cu:445-446, raw_vertices.cu:59,
// sensor_pose_estimation.cu:255-256; Mat operator* at sensor_pose_estimation.cu:343,428;
// cv::Cholesky at :399).  Here they run on the device inside the frame's kernels so
// that no host round trip is needed, restated from OpenCV's published algorithms:
//   inv3  -- closed-form adjugate, double products, one rounding to float
//   inv4  -- float LU with partial pivoting (cv::invert DECOMP_LU, hal::LU32f)
//   mat4  -- 4x4 product accumulated in double, rounded to float (cv::gemm)
//   chol6 -- in-place Cholesky with double accumulators and float storage of L,
//            reciprocal diagonal, forward/back substitution (hal::Cholesky32f);
//            returns false and leaves b untouched when a pivot is below FLT_EPSILON.
// Every file that includes this is compiled without FMA contraction (-fmad=false on
// the device, -ffp-contract=off on the host), so host and device give the same bits.
// Attribution: these algorithms are OpenCV's (https://opencv.org, Apache License 2.0),
// restated here; no OpenCV source is included.
#pragma once

#include <cfloat>
#include <cmath>

#if defined(__CUDACC__)
#define KF_HD __host__ __device__ __forceinline__
#else
#define KF_HD inline
#endif

namespace kf {

KF_HD void inv3(const float* m, float* out)
{
    double d = m[0] * ((double)m[4] * m[8] - (double)m[5] * m[7]) - m[1] * ((double)m[3] * m[8] - (double)m[5] * m[6]) +
               m[2] * ((double)m[3] * m[7] - (double)m[4] * m[6]);
    if (d == 0.0) {
        for (int i = 0; i < 9; ++i) out[i] = 0.f;
        return;
    }
    d = 1.0 / d;
    out[0] = (float)(((double)m[4] * m[8] - (double)m[5] * m[7]) * d);
    out[1] = (float)(((double)m[2] * m[7] - (double)m[1] * m[8]) * d);
    out[2] = (float)(((double)m[1] * m[5] - (double)m[2] * m[4]) * d);
    out[3] = (float)(((double)m[5] * m[6] - (double)m[3] * m[8]) * d);
    out[4] = (float)(((double)m[0] * m[8] - (double)m[2] * m[6]) * d);
    out[5] = (float)(((double)m[2] * m[3] - (double)m[0] * m[5]) * d);
    out[6] = (float)(((double)m[3] * m[7] - (double)m[4] * m[6]) * d);
    out[7] = (float)(((double)m[1] * m[6] - (double)m[0] * m[7]) * d);
    out[8] = (float)(((double)m[0] * m[4] - (double)m[1] * m[3]) * d);
}

KF_HD bool inv4(const float* src, float* out)
{
    float a[16], b[16];
    for (int i = 0; i < 16; ++i) {
        a[i] = src[i];
        b[i] = (i % 5 == 0) ? 1.f : 0.f;
    }
    const float eps = FLT_EPSILON * 10;
    for (int i = 0; i < 4; ++i) {
        int p = i;
        for (int j = i + 1; j < 4; ++j)
            if (fabsf(a[j * 4 + i]) > fabsf(a[p * 4 + i])) p = j;
        if (fabsf(a[p * 4 + i]) < eps) {
            for (int t = 0; t < 16; ++t) out[t] = 0.f;
            return false;
        }
        if (p != i) {
            for (int j = i; j < 4; ++j) {
                const float t = a[i * 4 + j];
                a[i * 4 + j] = a[p * 4 + j];
                a[p * 4 + j] = t;
            }
            for (int j = 0; j < 4; ++j) {
                const float t = b[i * 4 + j];
                b[i * 4 + j] = b[p * 4 + j];
                b[p * 4 + j] = t;
            }
        }
        const float d = -1 / a[i * 4 + i];
        for (int j = i + 1; j < 4; ++j) {
            const float alpha = a[j * 4 + i] * d;
            for (int c = i + 1; c < 4; ++c) a[j * 4 + c] += alpha * a[i * 4 + c];
            for (int c = 0; c < 4; ++c) b[j * 4 + c] += alpha * b[i * 4 + c];
        }
    }
    for (int i = 3; i >= 0; --i)
        for (int j = 0; j < 4; ++j) {
            float s = b[i * 4 + j];
            for (int c = i + 1; c < 4; ++c) s -= a[i * 4 + c] * b[c * 4 + j];
            b[i * 4 + j] = s / a[i * 4 + i];
        }
    for (int i = 0; i < 16; ++i) out[i] = b[i];
    return true;
}

#if defined(__CUDACC__)
// inv4 by one warp (all 32 lanes call), bit-identical to inv4: lane l holds entry
// (r, c) = (l >> 3, l & 7) of [a | b] (c < 4: a; c >= 4: b, the identity on entry), and
// every operation of inv4 on an entry is done by that entry's lane, in inv4's order:
// the pivot search runs the same compares in every lane, rows are swapped by shuffles,
// each elimination step is one product and one sum per lane, and the back substitution
// runs row by row with the four columns in parallel.  Writes out[0..15] from the lanes
// holding b (or zeros, and returns false, where inv4 would).
__device__ __forceinline__ bool inv4_warp(const float* src, float* out)
{
    const unsigned full = 0xffffffffu;
    const int l = threadIdx.x & 31, r = l >> 3, c = l & 7;
    float v = c < 4 ? src[r * 4 + c] : (c - 4 == r ? 1.f : 0.f);
    const float eps = FLT_EPSILON * 10;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float col[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) col[j] = __shfl_sync(full, v, j * 8 + i);
        int p = i;
        float best = col[i];
#pragma unroll
        for (int j = i + 1; j < 4; ++j)
            if (fabsf(col[j]) > fabsf(best)) {
                p = j;
                best = col[j];
            }
        if (fabsf(best) < eps) {  // the same in every lane
            if (l < 16) out[l] = 0.f;
            return false;
        }
        // rows i and p trade their a entries from column i on and all their b entries
        const int from = r == i ? p : (r == p ? i : r);
        const float other = __shfl_sync(full, v, from * 8 + c);
        if (from != r && (c >= 4 || c >= i)) v = other;
        const float d = -1 / __shfl_sync(full, v, i * 8 + i);
        const float aji = __shfl_sync(full, v, r * 8 + i);
        const float aic = __shfl_sync(full, v, i * 8 + c);
        if (r > i && (c >= 4 || c > i)) {
            const float alpha = aji * d;
            v += alpha * aic;
        }
    }
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        float s = v;
#pragma unroll
        for (int k = i + 1; k < 4; ++k) {
            const float aik = __shfl_sync(full, v, i * 8 + k);
            const float bkj = __shfl_sync(full, v, k * 8 + c);
            s -= aik * bkj;
        }
        const float aii = __shfl_sync(full, v, i * 8 + i);
        if (r == i && c >= 4) v = s / aii;
    }
    if (c >= 4) out[r * 4 + (c - 4)] = v;
    return true;
}

// entry (r, c) = (k >> 2, k & 3) of mat4(a, b)
__device__ __forceinline__ float mat4_at(const float* a, const float* b, int k)
{
    const int i = k >> 2, j = k & 3;
    double s = (double)a[i * 4 + 0] * b[j];
    s += (double)a[i * 4 + 1] * b[4 + j];
    s += (double)a[i * 4 + 2] * b[8 + j];
    s += (double)a[i * 4 + 3] * b[12 + j];
    return (float)s;
}
#endif

// out = a * b (out may alias a or b)
KF_HD void mat4(const float* a, const float* b, float* out)
{
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = (double)a[i * 4 + 0] * b[j];
            s += (double)a[i * 4 + 1] * b[4 + j];
            s += (double)a[i * 4 + 2] * b[8 + j];
            s += (double)a[i * 4 + 3] * b[12 + j];
            r[i * 4 + j] = (float)s;
        }
    for (int i = 0; i < 16; ++i) out[i] = r[i];
}

// A: 6x6 row-major, lower triangle read and overwritten; b: right-hand side -> solution
KF_HD bool chol6(float* A, float* b)
{
    const int m = 6;
    double s;
    int i, j, k;
    for (i = 0; i < m; ++i) {
        for (j = 0; j < i; ++j) {
            s = A[i * m + j];
            for (k = 0; k < j; ++k) s -= A[i * m + k] * A[j * m + k];
            A[i * m + j] = (float)(s * A[j * m + j]);
        }
        s = A[i * m + i];
        for (k = 0; k < j; ++k) {
            const double t = A[i * m + k];
            s -= t * t;
        }
        if (s < FLT_EPSILON) return false;
        A[i * m + i] = (float)(1. / sqrt(s));
    }
    for (i = 0; i < m; ++i) {
        s = b[i];
        for (k = 0; k < i; ++k) s -= A[i * m + k] * b[k];
        b[i] = (float)(s * A[i * m + i]);
    }
    for (i = m - 1; i >= 0; --i) {
        s = b[i];
        for (k = m - 1; k > i; --k) s -= A[k * m + i] * b[k];
        b[i] = (float)(s * A[i * m + i]);
    }
    return true;
}

// the small-angle increment of sensor_pose_estimation.cu:406-425,
// x = (beta, gamma, alpha, tx, ty, tz)
KF_HD void increment(const float* x, float* inc)
{
    inc[0] = 1.0f;  inc[1] = x[2];  inc[2] = -x[1]; inc[3] = x[3];
    inc[4] = -x[2]; inc[5] = 1.0f;  inc[6] = x[0];  inc[7] = x[4];
    inc[8] = x[1];  inc[9] = -x[0]; inc[10] = 1.0f; inc[11] = x[5];
    inc[12] = 0.0f; inc[13] = 0.0f; inc[14] = 0.0f; inc[15] = 1.0f;
}

#if defined(__CUDACC__)
// (float)(1. / sqrt(s)) for a double s -- the Cholesky pivot of hal::Cholesky32f --
// bit for bit, mostly without the FP64 square root and division (about 900 dependent
// cycles on a GPU with reduced FP64 throughput).  Ziv's strategy: an approximation
// with a proven error bound decides the float rounding unless it lies too close to a
// rounding boundary; only then is the exact FP64 expression evaluated.
//   y0 = rsqrtf((float)s)                      relative error <= 2^-24 + 2 ulp < 2^-21
//   e  = 1 - s*y0*y0   (y0*y0 exact in double; the product rounds by <= 2^-53; the
//                       subtraction is exact by Sterbenz since s*y0*y0 is near 1)
//   1/sqrt(s) = y0 (1 - e)^(-1/2) = y0 (1 + e/2 + 3e^2/8 + ...)
//   c  = y0 * (e/2) in float; y0 + c approximates 1/sqrt(s) within 2^-42 relative
//   (truncation 3e^2/8 < 2^-43, roundings of e and c < 2^-45 each).
// f = fl(y0 + c) and err = (y0 + c) - f exactly (Fast2Sum, |y0| > |c|).  The FP64
// expression is within 2^-52 of 1/sqrt(s), so when err keeps a margin of 2^-36 |f|
// from the half-gap to f's neighbour on its side, both round to f.
__device__ __forceinline__ float rsqrt_pivot(double s)
{
    if (s >= 1e-30 && s <= 1e30) {
        const float y0 = rsqrtf((float)s);
        const double y2 = (double)y0 * (double)y0;
        const double e = 1.0 - s * y2;
        if (fabs(e) < 0x1p-18) {
            const float c = y0 * (0.5f * (float)e);
            const float f = y0 + c;
            const float err = c - (f - y0);
            const int bits = __float_as_int(f);
            const float half_gap = err >= 0.f ? 0.5f * (__int_as_float(bits + 1) - f)
                                              : 0.5f * (f - __int_as_float(bits - 1));
            if (fabsf(err) + f * 0x1p-36f < half_gap) return f;
        }
    }
    return (float)(1. / sqrt(s));
}
#endif

}  // namespace kf
