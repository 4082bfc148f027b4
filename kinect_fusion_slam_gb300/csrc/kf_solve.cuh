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
// Attribution: cv::Cholesky's and cv::gemm's algorithms are OpenCV's (https://opencv.org,
// Apache License 2.0), restated here; no OpenCV source is included.
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
// Lane r (r + 1) / 2 + c holds entry (r, c) of the lower triangle as a running sum.
// The factor is computed column by column: column j's pivot and then its other entries
// are rounded from their sums, and every entry right of column j subtracts its term of
// column j at once (right-looking), so each entry's terms still come in chol6's order,
// k = 0, 1, ..., c - 1.  The substitutions likewise keep one row per lane: once x_k is
// final, every later row subtracts its term of x_k, each row's terms in chol6's order.
// Shared L keeps A's value in an entry until the entry is final (the FP64 fallbacks
// read both).
__device__ __forceinline__ bool warp_chol6(float* L, float* x, int* fail)
{
    const int lane = threadIdx.x & 31;
    const bool ent = lane < 21;
    const int r = (lane >= 1) + (lane >= 3) + (lane >= 6) + (lane >= 10) + (lane >= 15);
    const int c = ent ? lane - r * (r + 1) / 2 : 0;
    const int rr = ent ? r : 0;
    ff::Acc acc;
    acc.init(ent ? L[rr * 6 + c] : 0.f);
    if (lane == 0) *fail = 0;
    __syncwarp();
    for (int j = 0; j < 6; ++j) {
        if (ent && rr == j && c == j) {
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
        if (ent && c == j && rr > j) {
            const float piv = L[j * 6 + j];
            float v;
            if (!ff::mul_round_f32(acc.h, acc.l, acc.bound(), piv, v)) v = ff::offdiag_f64(L, rr, j);
            L[rr * 6 + j] = v;
        }
        __syncwarp();
        if (ent && c > j) {
            // the diagonal subtracts the exact square of L[r][j], the other entries the
            // float product L[r][j] * L[c][j]
            const float t = L[rr * 6 + j];
            const float u = rr == c ? t : L[c * 6 + j];
            const float pr = t * u;
            const float pe = rr == c ? fmaf(t, u, -pr) : 0.f;
            float sum, e;
            ff::two_sum(acc.h, -pr, sum, e);
            acc.h = sum;
            acc.l = (acc.l + e) - pe;
            acc.m = acc.m + fabsf(pr);
        }
    }
    // forward: row i = lane i
    const bool row = lane < 6;
    ff::Acc ax;
    ax.init(row ? x[lane] : 0.f);
    for (int k = 0; k < 6; ++k) {
        if (lane == k) {
            float v;
            if (!ff::mul_round_f32(ax.h, ax.l, ax.bound(), L[k * 6 + k], v)) v = ff::subst_f64(L, x, k, 0);
            x[k] = v;
        }
        __syncwarp();
        if (row && lane > k) ax.add(-(L[lane * 6 + k] * x[k]));
    }
    // backward
    ax.init(row ? x[lane] : 0.f);
    __syncwarp();
    for (int k = 5; k >= 0; --k) {
        if (lane == k) {
            float v;
            if (!ff::mul_round_f32(ax.h, ax.l, ax.bound(), L[k * 6 + k], v)) v = ff::subst_f64(L, x, k, 1);
            x[k] = v;
        }
        __syncwarp();
        if (row && lane < k) ax.add(-(L[k * 6 + lane] * x[k]));
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
// [2^-999, 2^1000).  y0 = rcp.approx.ftz.f64(p) has a relative error e0 = 1 - p y0
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

// Gauss-Jordan elimination of [A | b] in FP64 by one warp with IEEE divisions, for a
// symmetric A and without pivoting.  Lane c < 6 holds column c of A and lane 6 holds b
// (col[i] = row i); after the six steps lane 6 holds A^-1 b.  For a positive definite
// A the pivots are the successive Schur complements, all positive (the squares of the
// Cholesky factor's diagonal); a pivot that is not > 0 is Cholesky's failure test and
// the solve returns false (the same in every lane).  The fallback of pair_gj6_f64.
__device__ __forceinline__ bool warp_gj6_f64_ieee(double (&col)[6])
{
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

// bar.sync on a named barrier of the 64 threads of a warp pair
__device__ __forceinline__ void pair_bar(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }

// bar.red.or over the warp pair: true in every thread when any thread passes true
__device__ __forceinline__ bool pair_bar_or(int id, bool v)
{
    unsigned out;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, 64, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(out)
        : "r"((unsigned)v), "r"(id)
        : "memory");
    return out != 0u;
}

// v * 2^(1023 - e), e the exponent field of a normal pivot, by integer arithmetic on
// v's exponent field (exact where the result is normal).  Zero where v is zero or
// subnormal or the result would be subnormal (a term below 2^-1022 of the pivot row's
// scale); `over` is set where the result would overflow or v is not finite.  No branch.
__device__ __forceinline__ double scale_by_pivot(double v, int e, bool& over)
{
    const int hi = __double2hiint(v), lo = __double2loint(v);
    const int ev = (hi >> 20) & 0x7ff;
    const int en = ev - e + 1023;
    over = over || ev == 0x7ff || en > 2046;
    const double sc = __hiloint2double((hi & 0x800fffff) | ((en & 0x7ff) << 20), lo);
    return (ev == 0 || en < 1) ? 0.0 : sc;
}

// The precision form's 6x6 solve A x = b in FP64 by a pair of warps (the 64 threads
// t = threadIdx.x - 64 * pair of one warp pair call; named barriers bar_id and
// bar_id + 1 are the pair's: bar.sync on the first, bar.red on the second).  A is symmetric; entry(r, c) gives A[r][c] for c < 6 and b[r] for c == 6.
//
// This GPU retires one FP64 warp instruction per ~64 cycles per SM sub-partition, so
// the solve is laid out to put as few of them as possible on its critical path: one
// entry of [A | b] per thread (warp w holds rows 3w..3w+2, lane l < 21 the entry
// (3w + l / 7, l % 7)), exchanged through shared memory once per step, and
// fraction-free Gauss-Jordan steps, row_i <- p' row_i - m'_i row_j for i != j, where p
// is the pivot a_jj, m_i = a_ij, and p' = p 2^-E, m'_i = m_i 2^-E for E = exponent(p)
// (exact power-of-two scaling by integer arithmetic on the exponent field, which keeps
// the entries from growing like products of pivots).  Each step is one FP64 product
// and one FMA per thread, with no division.  Every row is thereby scaled by positive
// factors only, so the pivots have the signs of the Schur complements: a pivot that is
// not > 0 is Cholesky's failure test, and the solve returns false.  After the six
// steps the A part of row r is diagonal, and x_r = b'_r / a'_rr is one division per row
// (div_pivot).  A system whose pivots or scaled entries leave the normal range, or
// whose solution is not finite, is decided and solved again by warp_gj6_f64_ieee.
//
// Returns true (in all 64 threads) when A is positive definite; then x[0..5] (shared)
// holds the solution.  buf: 2 x 6 x 8 shared doubles of scratch.
template <class Entry>
__device__ __forceinline__ bool pair_gj6_f64(const Entry& entry, int t, double (*buf)[6][8], double* x, int bar_id)
{
    const int w = t >> 5, l = t & 31;
    const bool act = l < 21;
    const int r = act ? 3 * w + l / 7 : 0, c = act ? l % 7 : 0;
    double a = act ? entry(r, c) : 0.0;
    bool pd = true, bad = false;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double(*M)[8] = buf[j & 1];
        if (act) M[r][c] = a;
        pair_bar(bar_id);
        const double p = M[j][j];
        const int ep = (__double2hiint(p) >> 20) & 0x7ff;
        // p > 0 by its sign bit: a zero, subnormal or non-finite p (ep 0 or 0x7ff) sets
        // bad and is decided again below (comparisons run on the FP64 pipe here)
        pd = pd && __double2hiint(p) >= 0;
        bad = bad || ep == 0 || ep == 0x7ff;
        const double ps = scale_by_pivot(p, ep, bad);  // in [1, 2)
        // rows i != j: a <- p' a - m' q on the live columns c > j, a <- p' a elsewhere
        // (on the diagonal of a finished row, which scales with its row; the other
        // entries there are dead); row j stays.  Two FP64 operations in every lane,
        // without divergence.
        const double q = M[j][c];
        const double ms = (r != j && c > j) ? scale_by_pivot(M[r][j], ep, bad) : 0.0;
        a = fma(-ms, q, (r == j ? 1.0 : ps) * a);
    }
    // lane (r, 6) divides by the diagonal (r, r) of its row, held in the same warp
    const double d = __shfl_sync(0xffffffffu, a, act ? (l / 7) * 7 + r : 0);
    bool inf = false;
    if (act && c == 6) {
        // d in [2^-999, 2^1000) by its sign and exponent field
        const int dh = __double2hiint(d), ed = (dh >> 20) & 0x7ff;
        const double xr = (dh >= 0 && ed > 23 && ed < 2023) ? div_pivot(a, d) : a / d;
        inf = ((__double2hiint(xr) >> 20) & 0x7ff) == 0x7ff;
        x[r] = xr;
    }
    // out of range anywhere: neither the decision nor x can be trusted (a subnormal
    // pivot, say, scales to zero and makes the next pivot zero)
    if (!pair_bar_or(bar_id + 1, bad || (pd && inf))) return pd;  // also publishes x
    // rare: redo with IEEE divisions by the first warp; the second waits at the barrier
    bool fail = false;
    if (w == 0) {
        double col[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) col[i] = l < 7 ? entry(i, l) : 0.0;
        fail = !warp_gj6_f64_ieee(col);
        if (l == 6 && !fail)
#pragma unroll
            for (int i = 0; i < 6; ++i) x[i] = col[i];
    }
    return !pair_bar_or(bar_id + 1, fail && l == 0);
}

}  // namespace kf
