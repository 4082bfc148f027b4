/*
 * TEST INFRASTRUCTURE.  Lets the reference's CUDA kernel bodies compile unchanged as
 * host C++: CUDA qualifiers become nothing, float3 becomes a plain struct, and the
 * launch indices become thread-local variables set by the harness before each call.
 */
#ifndef KF_REF_SHIM_H
#define KF_REF_SHIM_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

using std::abs;
using std::acos;
using std::floor;
using std::isnan;

struct float3 {
    float x, y, z;
};
static inline float3 make_float3(float a, float b, float c) { return float3{a, b, c}; }

struct kf_ref_dim3 {
    unsigned x, y, z;
};
extern thread_local kf_ref_dim3 blockIdx, threadIdx, blockDim;

/* raycast hit recorder inserted by the splice recipe after the first output write */
extern thread_local int32_t* kf_ref_hit_plane;
#define KF_REF_HIT(px, vi)                                  \
    do {                                                    \
        if (kf_ref_hit_plane) kf_ref_hit_plane[px] = (vi); \
    } while (0)

#define __global__
#define __device__
#define __forceinline__ inline
#define CUDART_PI_F 3.141592654f

#endif
