// The ICP pose update of one iteration (cv::Cholesky at sensor_pose_estimation.cu:399
// and the two cv::Mat products at :343 and :428) for one warp, bit-identical to the
// FP64 restatements chol6 and mat4 of kf_math.cuh, mostly in FP32.
//
// Those restatements accumulate in double: every entry is a short sequence
// s <- RN64(s + d) over exact terms d (floats, or products of two floats, which a
// double holds exactly), and the result is rounded to float, possibly after one more
// double product or a reciprocal square root.  This GPU's FP64 unit takes 64-150
// cycles per dependent instruction, about 20 times its FP32 latency, and a Cholesky
// solve is a long chain of them.  So each sum is carried instead as an unevaluated
// pair of floats h + l (error-free TwoSum for the running sum, the rounding errors
// collected in l) together with m, the sum of the terms' magnitudes.  With n <= 7
// terms, h + l lies within 2^-40.7 m of the exact sum, and the reference's double
// within another n 2^-53 m, so both lie within E = 2^-39 m of h + l.  The float result
// is decided by Ziv's test: if h + l rounds to f and stays more than E away from the
// midpoints between f and its neighbours, the double rounds to f as well.  Otherwise
// (about one entry in 10^4 on random systems, more under heavy cancellation) the entry
// is recomputed by the FP64 sequence itself.  Every file that includes this is
// compiled with -fmad=false, so the float expressions below are evaluated as written.
#pragma once

#include <cfloat>

#include "kf_math.cuh"

namespace kf {
namespace ff {

// s = RN(a + b) and e = a + b - s exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// A double-accumulated sum carried as h + l, with m = sum of the terms' magnitudes.
struct Acc {
    float h, l, m;
    __device__ __forceinline__ void init(float x)
    {
        h = x;
        l = 0.f;
        m = fabsf(x);
    }
    __device__ __forceinline__ void init_prod(float x, float y)
    {
        h = x * y;
        l = fmaf(x, y, -h);  // exact: the product's rounding error
        m = fabsf(h);
    }
    // += x, x a float
    __device__ __forceinline__ void add(float x)
    {
        float s, e;
        two_sum(h, x, s, e);
        h = s;
        l = l + e;
        m = m + fabsf(x);
    }
    // += x * y exactly (the double product of two floats)
    __device__ __forceinline__ void add_prod(float x, float y)
    {
        const float p = x * y;
        const float pe = fmaf(x, y, -p);
        float s, e;
        two_sum(h, p, s, e);
        h = s;
        l = (l + e) + pe;
        m = m + fabsf(p);
    }
    // distance within which the reference's double lies from h + l
    __device__ __forceinline__ float bound() const { return m * 0x1p-39f; }
};

// the float next to |a| on the side of r (away from zero when r has a's sign)
__device__ __forceinline__ float half_gap(float f, float r)
{
    const float a = fabsf(f);
    const int bits = __float_as_int(a);
    const float away = f > 0.f ? r : -r;
    return away >= 0.f ? 0.5f * (__int_as_float(bits + 1) - a) : 0.5f * (a - __int_as_float(bits - 1));
}

__device__ __forceinline__ bool normal_range(float a) { return a >= 0x1p-100f && a <= 0x1p100f; }

// RN32 of a double d with |d - (h + l)| <= E; false when that is not decided
__device__ __forceinline__ bool round_f32(float h, float l, float E, float& out)
{
    if (E == 0.f) {  // every term was a zero: h is the double's signed zero
        out = h;
        return true;
    }
    float f, r;
    two_sum(h, l, f, r);
    if (!normal_range(fabsf(f))) return false;
    if (fabsf(r) + E < half_gap(f, r)) {
        out = f;
        return true;
    }
    return false;
}

// RN32(RN64(d * m)) for a float m and a double d with |d - (h + l)| <= E
__device__ __forceinline__ bool mul_round_f32(float h, float l, float E, float m, float& out)
{
    if (E == 0.f) {
        out = h * m;
        return true;
    }
    float H, L;
    two_sum(h, l, H, L);  // |L| <= 2^-24 |H|
    const float ph = H * m;
    const float pe = fmaf(H, m, -ph);
    const float pl = pe + L * m;
    // d m is within E|m| of (H + L) m = ph + pe + L m; the two roundings in pl and the
    // double product's own rounding add less than 2^-44 |ph|
    return round_f32(ph, pl, E * fabsf(m) + fabsf(ph) * 0x1p-44f, out);
}

// RN32(RN64(1 / RN64(sqrt(d)))) for a double d with |d - (h + l)| <= E and d >= FLT_EPSILON.
// y0 = rsqrtf(H) and e = 1 - (H + L) y0^2 (y0^2 and H y0h exact by FMA, the rest below
// 2^-41 absolute); 1/sqrt(H + L) = y0 (1 + e/2 + 3e^2/8 + ...) is approximated by
// y0 + y0 e/2 within 2^-37 relative for |e| < 2^-18; d's distance from H + L moves the
// result by E/(2d) relative and the double roundings by 2^-52.
__device__ __forceinline__ bool rsqrt_round_f32(float h, float l, float E, float& out)
{
    float H, L;
    two_sum(h, l, H, L);
    if (!(H >= 0x1p-60f && H <= 0x1p60f) || !(E <= H * 0x1p-20f)) return false;
    const float y0 = rsqrtf(H);
    const float y2h = y0 * y0;
    const float y2l = fmaf(y0, y0, -y2h);
    const float ph = H * y2h;
    const float pe = fmaf(H, y2h, -ph);
    const float pl = pe + (H * y2l + L * y2h);
    const float e = (1.f - ph) - pl;
    if (!(fabsf(e) < 0x1p-18f)) return false;
    const float c = y0 * (0.5f * e);
    float f, r;
    two_sum(y0, c, f, r);
    if (fabsf(r) + f * (0x1p-36f + E / H) < half_gap(f, r)) {
        out = f;
        return true;
    }
    return false;
}

// The FP64 sequences of chol6 for one entry, used when the float test above does not
// decide it.  Out of line, so the compiler keeps them behind a branch instead of
// issuing their FP64 instructions under a predicate on every call.
// pivot of row j: sets *fail or L[j][j]
static __device__ __noinline__ void pivot_f64(float* L, int j, int* fail)
{
    double sd = L[j * 6 + j];
    for (int k = 0; k < j; ++k) {
        const double t = L[j * 6 + k];
        sd -= t * t;
    }
    if (sd < FLT_EPSILON)
        *fail = 1;
    else
        L[j * 6 + j] = rsqrt_pivot(sd);
}

// off-diagonal entry (i, j) of the factor from A[i][j]
static __device__ __noinline__ float offdiag_f64(const float* L, int i, int j)
{
    double sd = L[i * 6 + j];
    for (int k = 0; k < j; ++k) sd -= L[i * 6 + k] * L[j * 6 + k];
    return (float)(sd * L[j * 6 + j]);
}

// forward (dir 0) or backward (dir 1) substitution entry i
static __device__ __noinline__ float subst_f64(const float* L, const float* x, int i, int dir)
{
    double sd = x[i];
    if (dir == 0)
        for (int k = 0; k < i; ++k) sd -= L[i * 6 + k] * x[k];
    else
        for (int k = 5; k > i; --k) sd -= L[k * 6 + i] * x[k];
    return (float)(sd * L[i * 6 + i]);
}

// entry (r, c) of mat4(a, b)
static __device__ __noinline__ float mat4_entry_f64(const float* a, const float* b, int r, int c)
{
    double s = (double)a[r * 4 + 0] * b[c];
    s += (double)a[r * 4 + 1] * b[4 + c];
    s += (double)a[r * 4 + 2] * b[8 + c];
    s += (double)a[r * 4 + 3] * b[12 + c];
    return (float)s;
}

}  // namespace ff

// The Cholesky solve of chol6 by the calling warp (all 32 lanes call).  L: 6x6 shared,
// lower triangle holding A on entry and the factor (reciprocal diagonal) on return;
// x: 6 shared floats, b on entry, the solution on return when the factorisation
// succeeds and untouched when a pivot is below FLT_EPSILON (then false is returned).
// The factor is computed column by column -- column j's pivot by lane j, its other
// entries by lanes j+1..5 -- with each entry's terms in chol6's order.
__device__ __forceinline__ bool warp_chol6(float* L, float* x, int* fail)
{
    const int lane = threadIdx.x & 31;
    if (lane == 0) *fail = 0;
    __syncwarp();
    for (int j = 0; j < 6; ++j) {
        const int row = lane < 6 ? lane : 5;
        const bool active = lane >= j && lane < 6;
        ff::Acc acc;
        acc.init(active ? L[row * 6 + j] : 0.f);
        if (active) {
            for (int k = 0; k < j; ++k) {
                // the pivot subtracts the exact square of L[j][k], the other entries the
                // float product L[row][k] * L[j][k]; one instruction stream for both
                const float t = L[row * 6 + k];
                const float u = lane == j ? t : L[j * 6 + k];
                const float p = t * u;
                const float pe = lane == j ? fmaf(t, u, -p) : 0.f;
                float s, e;
                ff::two_sum(acc.h, -p, s, e);
                acc.h = s;
                acc.l = (acc.l + e) - pe;
                acc.m = acc.m + fabsf(p);
            }
        }
        if (lane == j) {
            const float H = acc.h + acc.l, E = acc.bound();
            bool decided = false;
            if (H * 0.999f - 2.f * E >= FLT_EPSILON) {
                float piv;
                if (ff::rsqrt_round_f32(acc.h, acc.l, E, piv)) {
                    L[j * 6 + j] = piv;
                    decided = true;
                }
            } else if (H * 1.001f + 2.f * E < FLT_EPSILON) {
                *fail = 1;
                decided = true;
            }
            if (!decided) ff::pivot_f64(L, j, fail);
        }
        __syncwarp();
        if (*fail) return false;
        if (lane > j && lane < 6) {
            const float piv = L[j * 6 + j];
            float v;
            if (!ff::mul_round_f32(acc.h, acc.l, acc.bound(), piv, v)) v = ff::offdiag_f64(L, lane, j);
            L[lane * 6 + j] = v;
        }
        __syncwarp();
    }
    if (lane == 0) {
        for (int i = 0; i < 6; ++i) {
            ff::Acc acc;
            acc.init(x[i]);
            for (int k = 0; k < i; ++k) acc.add(-(L[i * 6 + k] * x[k]));
            float v;
            if (!ff::mul_round_f32(acc.h, acc.l, acc.bound(), L[i * 6 + i], v)) v = ff::subst_f64(L, x, i, 0);
            x[i] = v;
        }
        for (int i = 5; i >= 0; --i) {
            ff::Acc acc;
            acc.init(x[i]);
            for (int k = 5; k > i; --k) acc.add(-(L[k * 6 + i] * x[k]));
            float v;
            if (!ff::mul_round_f32(acc.h, acc.l, acc.bound(), L[i * 6 + i], v)) v = ff::subst_f64(L, x, i, 1);
            x[i] = v;
        }
    }
    __syncwarp();
    return true;
}

// entry (r, c) = (lane >> 2, lane & 3) of mat4(a, b), for lanes 0..15
__device__ __forceinline__ float mat4_entry(const float* a, const float* b, int lane)
{
    const int r = lane >> 2, c = lane & 3;
    ff::Acc acc;
    acc.init_prod(a[r * 4 + 0], b[c]);
    acc.add_prod(a[r * 4 + 1], b[4 + c]);
    acc.add_prod(a[r * 4 + 2], b[8 + c]);
    acc.add_prod(a[r * 4 + 3], b[12 + c]);
    float v;
    if (ff::round_f32(acc.h, acc.l, acc.bound(), v)) return v;
    return ff::mat4_entry_f64(a, b, r, c);
}

// Division by the pivot in the Gauss-Jordan steps: q = a / p for p > 0 in
// [2^-1000, 2^1000].  y0 = rcp.approx.ftz.f64(p) has a relative error e0 = 1 - p y0
// of about 2^-20 (kf_selftest_solve6 checks the solves built on this); then
// a / p = a y0 / (1 - e0) = a y0 (1 + e0 + e0^2 + e0^3 + ...), and the first three terms
// leave a relative error e0^3 ~ 2^-60, below FP64 rounding.  a y0 and e0 are independent,
// so the dependent chain is the approximation and three FP64 operations (FP64 latency
// is ~64 cycles per operation on this part).
__device__ __forceinline__ double div_pivot(double a, double p)
{
    double y0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(p));
    const double q0 = a * y0;
    const double e0 = fma(-p, y0, 1.0);
    const double t = fma(e0, e0, e0);
    return fma(q0, t, q0);
}

// The precision form's solve: A x = b in FP64 by the calling warp (all 32 lanes call)
// for a symmetric A, by Gauss-Jordan elimination of [A | b] without pivoting.  For a
// positive definite A the pivots are the successive Schur complements, all positive
// (they are the squares of the Cholesky factor's diagonal); a pivot that is not > 0 is
// Cholesky's failure test, and the solve reports false.  Lane c < 6 holds column c of A
// and lane 6 holds b (col[i] = row i); after the six steps lane 6 holds A^-1 b.  The
// steps run without a branch (a step's critical path is the pivot's shuffle, its
// division and one update); the pivots are checked afterwards, and the rare system
// whose pivots fall outside div_pivot's range is solved again with IEEE divisions.
__device__ __forceinline__ bool warp_gj6_f64(double (&col)[6])
{
    double in[6], piv[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) in[i] = col[i];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const double p = __shfl_sync(0xffffffffu, col[j], j);
        piv[j] = p;
        double m[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) m[i] = __shfl_sync(0xffffffffu, col[i], j);
        const double aj = div_pivot(col[j], p);
#pragma unroll
        for (int i = 0; i < 6; ++i)
            if (i != j) col[i] = fma(-m[i], aj, col[i]);
        col[j] = aj;
    }
    bool pd = true, in_range = true;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        pd = pd && piv[j] > 0.0;
        in_range = in_range && piv[j] > 0x1p-1000 && piv[j] < 0x1p1000;
    }
    if (!pd) return false;  // the same in every lane
    if (in_range) return true;
#pragma unroll
    for (int i = 0; i < 6; ++i) col[i] = in[i];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const double p = __shfl_sync(0xffffffffu, col[j], j);
        if (!(p > 0.0)) return false;
        double m[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) m[i] = __shfl_sync(0xffffffffu, col[i], j);
        const double aj = col[j] / p;
#pragma unroll
        for (int i = 0; i < 6; ++i)
            if (i != j) col[i] = fma(-m[i], aj, col[i]);
        col[j] = aj;
    }
    return true;
}

}  // namespace kf
