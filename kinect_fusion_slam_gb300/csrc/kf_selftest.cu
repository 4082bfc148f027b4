// kf_selftest_solve: the float-float Cholesky solve and 4x4 product of kf_solve.cuh
// (warp_chol6, mat4_entry), which the ICP's pose update uses, against their FP64
// restatements chol6 and mat4 of kf_math.cuh, bit for bit, on seeded random systems.
// The systems are sums of rows a = (v x n, n) with v up to a few metres and unit n --
// the shape of the ICP's normal equations -- over 3 to 400 rows, so some are singular.
#include <cstdint>

#include "kinfu_gb300.h"
#include "kf_solve.cuh"

namespace {

constexpr int kWarps = 4;

__device__ __forceinline__ uint64_t mix(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ float uniform(uint64_t& s)
{
    s = mix(s + 0x9e3779b97f4a7c15ULL);
    return (float)((s >> 40) * 0x1p-24) * 2.f - 1.f;
}

// counts: systems, solve differences, factorisation-outcome differences, systems the
// FP64 restatement found not positive definite, 4x4 product entry differences
__global__ void __launch_bounds__(kWarps * 32) selftest_kernel(uint64_t seed, int per_warp,
                                                               unsigned long long* counts)
{
    __shared__ float L[kWarps][36], x[kWarps][6], Ar[kWarps][36], br[kWarps][6];
    __shared__ float ma[kWarps][16], mb[kWarps][16], mr[kWarps][16];
    __shared__ int fail[kWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long n = 0, bad = 0, badok = 0, fails = 0, badm = 0;
    for (int it = 0; it < per_warp; ++it) {
        uint64_t s = seed ^ ((blockIdx.x * (uint64_t)kWarps + w) * 1000003ULL + it) * 0x2545F4914F6CDD1DULL;
        if (lane == 0) {
            const int rows[6] = {3, 5, 6, 8, 64, 400};
            const int N = rows[mix(s) % 6];
            const float scale = 1.f + 3000.f * (0.5f + 0.5f * uniform(s));
            float A[36] = {}, b[6] = {};
            for (int r = 0; r < N; ++r) {
                const float v[3] = {scale * uniform(s), scale * uniform(s), scale * (1.5f + 0.5f * uniform(s))};
                float m[3] = {uniform(s), uniform(s), uniform(s)};
                const float inv = rsqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + 1e-12f);
                for (int k = 0; k < 3; ++k) m[k] *= inv;
                const float a[6] = {v[2] * m[1] - v[1] * m[2], -v[2] * m[0] + v[0] * m[2], v[1] * m[0] - v[0] * m[1],
                                    m[0], m[1], m[2]};
                const float rb = 20.f * uniform(s);
                for (int i = 0; i < 6; ++i) {
                    b[i] = b[i] + a[i] * rb;
                    for (int j = 0; j <= i; ++j) A[i * 6 + j] = A[i * 6 + j] + a[i] * a[j];
                }
            }
            for (int i = 0; i < 6; ++i) {
                br[w][i] = b[i];
                x[w][i] = b[i];
                for (int j = 0; j <= i; ++j) Ar[w][i * 6 + j] = L[w][i * 6 + j] = A[i * 6 + j];
            }
            for (int k = 0; k < 16; ++k) {
                ma[w][k] = (k % 5 == 0 ? 1.f : 0.f) + 0.05f * uniform(s);
                mb[w][k] = (k % 5 == 0 ? 1.f : 0.f) + ((k % 4 == 3 && k < 12) ? 1000.f * uniform(s) : 0.f);
            }
            if (mix(s) % 7 == 0) {
                ma[w][12] = ma[w][13] = ma[w][14] = 0.f;
                ma[w][15] = 1.f;
            }
        }
        __syncwarp();
        const bool ok = kf::warp_chol6(L[w], x[w], &fail[w]);
        const float mv = lane < 16 ? kf::mat4_entry(ma[w], mb[w], lane) : 0.f;
        __syncwarp();
        if (lane == 0) {
            const bool okr = kf::chol6(Ar[w], br[w]);
            kf::mat4(ma[w], mb[w], mr[w]);
            ++n;
            badok += ok != okr;
            fails += !okr;
            if (ok && okr) {
                bool diff = false;
                for (int i = 0; i < 6; ++i) {
                    diff |= __float_as_int(x[w][i]) != __float_as_int(br[w][i]);
                    for (int j = 0; j <= i; ++j) diff |= __float_as_int(L[w][i * 6 + j]) != __float_as_int(Ar[w][i * 6 + j]);
                }
                bad += diff;
            }
        }
        __syncwarp();
        if (lane < 16 && __float_as_int(mv) != __float_as_int(mr[w][lane])) ++badm;
        __syncwarp();
    }
    atomicAdd(&counts[0], n);
    atomicAdd(&counts[1], bad);
    atomicAdd(&counts[2], badok);
    atomicAdd(&counts[3], fails);
    atomicAdd(&counts[4], badm);
}

// one warp pair per system (pair_gj6_f64), two pairs per block on named barriers 1, 2
// and 3, 4
__global__ void __launch_bounds__(kWarps * 32) solve6_kernel(const double* __restrict__ A,
                                                             const double* __restrict__ b, double* __restrict__ x,
                                                             int* __restrict__ ok, int n)
{
    static_assert(kWarps == 4, "two warp pairs per block");
    __shared__ double buf[2][2][6][8], xs[2][6];
    const int pr = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int sys = blockIdx.x * 2 + pr;
    if (sys >= n) return;  // the same in the whole pair
    const double* As = A + (size_t)sys * 36;
    const double* bs = b + (size_t)sys * 6;
    const auto entry = [As, bs](int r, int c) { return c == 6 ? bs[r] : As[r * 6 + c]; };
    const bool solved = kf::pair_gj6_f64(entry, t, buf[pr], xs[pr], 1 + 2 * pr);
    if (t < 6 && solved) x[(size_t)sys * 6 + t] = xs[pr][t];
    if (t == 0) ok[sys] = solved ? 1 : 0;
}

}  // namespace

extern "C" kf_status kf_selftest_solve6(const double* A, const double* b, double* x, int* ok, int n)
{
    if (!A || !b || !x || !ok || n <= 0 || n > (1 << 20)) return KF_ERR_INVALID_ARGUMENT;
    double* d = nullptr;
    const size_t nd = (size_t)n * (36 + 6 + 6);
    if (cudaMalloc(&d, nd * sizeof(double) + (size_t)n * sizeof(int)) != cudaSuccess) return KF_ERR_CUDA;
    double *dA = d, *db = d + (size_t)n * 36, *dx = db + (size_t)n * 6;
    int* dok = (int*)(d + nd);
    cudaError_t e = cudaMemcpy(dA, A, (size_t)n * 36 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, b, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        solve6_kernel<<<(n + 1) / 2, kWarps * 32>>>(dA, db, dx, dok, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(x, dx, (size_t)n * 6 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ok, dok, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}

extern "C" kf_status kf_selftest_solve(unsigned long long seed, int blocks, int systems_per_warp,
                                       unsigned long long counts[5])
{
    if (!counts || blocks <= 0 || blocks > 65535 || systems_per_warp <= 0 || systems_per_warp > 4096)
        return KF_ERR_INVALID_ARGUMENT;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 5 * sizeof(unsigned long long)) != cudaSuccess) return KF_ERR_CUDA;
    cudaError_t e = cudaMemset(d, 0, 5 * sizeof(unsigned long long));
    if (e == cudaSuccess) {
        selftest_kernel<<<blocks, kWarps * 32>>>(seed, systems_per_warp, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(counts, d, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}
