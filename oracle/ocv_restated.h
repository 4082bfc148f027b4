/*
 * TEST INFRASTRUCTURE -- part of the CPU oracle, never linked into the product.
 *
 * Restatement of the four OpenCV (>= 4.1, CMakeLists.txt:10 of the reference; the
 * exact version is not pinned there) routines that the reference's per-frame path
 * calls on the host.  OpenCV is not present in this environment, so these follow
 * OpenCV's published algorithms (modules/core/src/matrix_decomp.cpp, lapack.cpp,
 * matmul.dispatch.cpp) as restated code:
 *
 *   ocv_inv3      cv::Mat::inv() of a 3x3 CV_32F matrix: closed-form adjugate with
 *                 double products and a double reciprocal determinant, rounded to
 *                 float once.  Called at raw_vertices.cu:59, projective_tsdf.cu:148,
 *                 voxel_traversal.cu:445, sensor_pose_estimation.cu:255.
 *   ocv_inv4      cv::Mat::inv() of a 4x4 CV_32F matrix: DECOMP_LU, i.e. float LU
 *                 with partial pivoting (hal::LU32f) solving A X = I.
 *                 Called at projective_tsdf.cu:149, voxel_traversal.cu:446,
 *                 sensor_pose_estimation.cu:256.
 *   ocv_matmul4   cv::Mat operator* on two 4x4 CV_32F matrices (gemm), accumulated in
 *                 double and rounded to float.  sensor_pose_estimation.cu:343,428.
 *   ocv_cholesky  cv::Cholesky(float*, ..., m=6, b, n=1): in-place Cholesky with
 *                 double accumulators, float storage of L (reciprocal diagonal), then
 *                 forward/back substitution.  Returns 0 (and leaves b untouched) when
 *                 a pivot falls below FLT_EPSILON.  sensor_pose_estimation.cu:399.
 *
 * Attribution: the algorithms restated here are OpenCV's (https://opencv.org,
 * Apache License 2.0); no OpenCV source is included.
 *
 * Parity for these four pieces is unpinned: no OpenCV build exists here to test
 * against.  The product restates the same algorithms independently in
 * kinect_fusion_slam_gb300/csrc/kf_math.cuh, and the tests check the two agree
 * bit for bit.
 */
#ifndef KF_ORACLE_OCV_RESTATED_H
#define KF_ORACLE_OCV_RESTATED_H

#include <cfloat>
#include <cmath>

static inline void ocv_inv3(const float* m, float* out)
{
    /* determinant expanded along the first row, products in double */
    double d = m[0] * ((double)m[4] * m[8] - (double)m[5] * m[7])
             - m[1] * ((double)m[3] * m[8] - (double)m[5] * m[6])
             + m[2] * ((double)m[3] * m[7] - (double)m[4] * m[6]);
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

/* float LU with partial pivoting on [A | I]; returns 0 when singular */
static inline int ocv_inv4(const float* src, float* out)
{
    float a[16], b[16];
    for (int i = 0; i < 16; ++i) { a[i] = src[i]; b[i] = (i % 5 == 0) ? 1.f : 0.f; }
    const float eps = FLT_EPSILON * 10;
    for (int i = 0; i < 4; ++i) {
        int k = i;
        for (int j = i + 1; j < 4; ++j)
            if (std::fabs(a[j * 4 + i]) > std::fabs(a[k * 4 + i])) k = j;
        if (std::fabs(a[k * 4 + i]) < eps) {
            for (int t = 0; t < 16; ++t) out[t] = 0.f;
            return 0;
        }
        if (k != i) {
            for (int j = i; j < 4; ++j) { float t = a[i * 4 + j]; a[i * 4 + j] = a[k * 4 + j]; a[k * 4 + j] = t; }
            for (int j = 0; j < 4; ++j) { float t = b[i * 4 + j]; b[i * 4 + j] = b[k * 4 + j]; b[k * 4 + j] = t; }
        }
        float d = -1 / a[i * 4 + i];
        for (int j = i + 1; j < 4; ++j) {
            float alpha = a[j * 4 + i] * d;
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
    return 1;
}

static inline void ocv_matmul4(const float* a, const float* b, float* out)
{
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = (double)a[i * 4 + 0] * b[0 * 4 + j];
            s += (double)a[i * 4 + 1] * b[1 * 4 + j];
            s += (double)a[i * 4 + 2] * b[2 * 4 + j];
            s += (double)a[i * 4 + 3] * b[3 * 4 + j];
            r[i * 4 + j] = (float)s;
        }
    for (int i = 0; i < 16; ++i) out[i] = r[i];
}

/* A: 6x6 row-major (lower triangle read, overwritten), b: 6 values (overwritten with x) */
static inline int ocv_cholesky6(float* A, float* b)
{
    const int m = 6;
    float* L = A;
    double s;
    int i, j, k;
    for (i = 0; i < m; ++i) {
        for (j = 0; j < i; ++j) {
            s = A[i * m + j];
            for (k = 0; k < j; ++k) s -= L[i * m + k] * L[j * m + k];
            L[i * m + j] = (float)(s * L[j * m + j]);
        }
        s = A[i * m + i];
        for (k = 0; k < j; ++k) {
            double t = L[i * m + k];
            s -= t * t;
        }
        if (s < FLT_EPSILON) return 0;
        L[i * m + i] = (float)(1. / std::sqrt(s));
    }
    for (i = 0; i < m; ++i) {
        s = b[i];
        for (k = 0; k < i; ++k) s -= L[i * m + k] * b[k];
        b[i] = (float)(s * L[i * m + i]);
    }
    for (i = m - 1; i >= 0; --i) {
        s = b[i];
        for (k = m - 1; k > i; --k) s -= L[k * m + i] * b[k];
        b[i] = (float)(s * L[i * m + i]);
    }
    for (i = 0; i < m; ++i) L[i * m + i] = 1 / L[i * m + i];
    return 1;
}

#endif
