// How far a pose's rotation block is from orthonormal: the largest |(R^T R - I)_ij| over
// the 3x3 block of a row-major 4x4 float pose.  Integration's box marks bound a voxel's
// camera depth by its distance from the camera, and its depth band through the length
// of its pixel's ray, both of which a rotation preserves; their margins (0.1 % on the
// band, 1 % on the distance) cover a deviation up to 5e-4.  The tracker's composed float
// poses drift by about 1e-9 per frame (a float simulation of Inc * T: 4.8e-5 after
// 50 000 frames, 3.3e-4 after 400 000), so beyond kRigidTol -- hours of tracking without
// a reset, or a scaled or sheared matrix given to kf_set_pose -- every box is listed
// instead (exact, at a dense pass's cost).  A NaN entry is skipped by fmaxf (a NaN pose
// updates nothing and lists nothing); an infinite one gives infinity.  Host and device
// code share it.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define KF_RIGID_HD __host__ __device__
#else
#define KF_RIGID_HD
#endif

namespace kf {

constexpr float kRigidTol = 2e-4f;

KF_RIGID_HD inline float rigid_error(const float* T)
{
    float e = 0.f;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) {
            const float d = T[i] * T[j] + T[4 + i] * T[4 + j] + T[8 + i] * T[8 + j] - (i == j ? 1.f : 0.f);
            e = fmaxf(e, fabsf(d));
        }
    return e;
}

}  // namespace kf
