// Division of a non-negative int by a run-time invariant divisor as a multiply-high and
// a shift (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, theorem 4.2, with N = 31): for 2 <= d < 2^31 let
// l = ceil(log2 d) and m = ceil(2^(31+l) / d).  Then 2^(31+l) <= m d < 2^(31+l) + 2^l,
// m < 2^32, and floor(n / d) = floor(n m / 2^(31+l)) = mulhi32(n, m) >> (l - 1) for every
// 0 <= n < 2^31.  Host and device code share it; the host computes the constants once.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define KF_DIVMAGIC_HD __host__ __device__
#else
#define KF_DIVMAGIC_HD
#endif

namespace kf {

struct DivMagic {
    uint32_t m;
    int s;
};

// d >= 2
inline DivMagic div_magic(uint32_t d)
{
    int l = 0;
    while ((1ull << l) < d) ++l;
    const uint64_t m = ((1ull << (31 + l)) + d - 1) / d;
    return DivMagic{(uint32_t)m, l - 1};
}

// floor(n / d) for 0 <= n < 2^31, q = div_magic(d)
KF_DIVMAGIC_HD inline int div_by(int n, DivMagic q)
{
#if defined(__CUDA_ARCH__)
    return (int)(__umulhi((unsigned)n, q.m) >> q.s);
#else
    return (int)((uint32_t)(((uint64_t)(uint32_t)n * q.m) >> 32) >> q.s);
#endif
}

}  // namespace kf
