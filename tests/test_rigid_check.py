"""Integration's box marks assume a rigid pose; kf_rigid.h's rigid_error (shared by host
and device) decides when a pose is too far from one and every box is listed instead.
Its host form is compiled here with g++ and checked: float rotations read as rigid,
scaled and sheared matrices do not, and 20 000 frames of float pose composition (the
tracker's Inc * T with float increments of up to ~1 degree) stay within a quarter of
the tolerance (measured 2.3e-5)."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "kinect_fusion_slam_gb300" / "csrc"

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include "kf_rigid.h"

static uint64_t state = 0x2545f4914f6cdd1dull;
static double uni()  // [-1, 1)
{
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (double)(state >> 11) / 4503599627370496.0 - 1.0;
}

// rotation by angle a about a random axis, with translation t, rounded to float
static void pose(double a, double tscale, float* T)
{
    double x = uni(), y = uni(), z = uni();
    const double n = std::sqrt(x * x + y * y + z * z) + 1e-300;
    x /= n; y /= n; z /= n;
    const double c = std::cos(a), s = std::sin(a), C = 1 - c;
    const double R[9] = {c + x * x * C, x * y * C - z * s, x * z * C + y * s,
                         y * x * C + z * s, c + y * y * C, y * z * C - x * s,
                         z * x * C - y * s, z * y * C + x * s, c + z * z * C};
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) T[4 * r + k] = (float)R[3 * r + k];
        T[4 * r + 3] = (float)(tscale * uni());
    }
    T[12] = T[13] = T[14] = 0.f;
    T[15] = 1.f;
}

static void mul(const float* A, const float* B, float* C)
{
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            float s = 0.f;
            for (int k = 0; k < 4; ++k) s = s + A[4 * r + k] * B[4 * k + c];
            C[4 * r + c] = s;
        }
}

int main()
{
    float T[16];
    float worst = 0.f;
    for (int k = 0; k < 100000; ++k) {
        pose(3.14159 * uni(), 50000.0, T);
        worst = std::fmax(worst, kf::rigid_error(T));
    }
    std::printf("random float rotations: %.3g\n", worst);
    if (!(worst < 1e-6f)) return 1;

    pose(0.7, 1000.0, T);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) T[4 * r + c] *= 1.001f;
    std::printf("scaled by 1.001: %.3g\n", kf::rigid_error(T));
    if (!(kf::rigid_error(T) > kf::kRigidTol)) return 2;

    pose(0.7, 1000.0, T);
    T[1] += 1e-3f;
    std::printf("sheared by 1e-3: %.3g\n", kf::rigid_error(T));
    if (!(kf::rigid_error(T) > kf::kRigidTol)) return 3;

    pose(0.7, 1000.0, T);
    T[5] = INFINITY;
    if (!(kf::rigid_error(T) > kf::kRigidTol)) return 4;

    // the tracker composes T <- Inc * T in float every frame
    float P[16], Q[16], I[16];
    pose(0.3, 1000.0, P);
    float drift = 0.f;
    for (int f = 0; f < 20000; ++f) {
        pose(0.02 * uni(), 20.0, I);
        mul(I, P, Q);
        for (int k = 0; k < 16; ++k) P[k] = Q[k];
        drift = std::fmax(drift, kf::rigid_error(P));
    }
    std::printf("20000 composed frames: %.3g\n", drift);
    if (!(drift < 0.25f * kf::kRigidTol)) return 5;
    return 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("rigid")
    src, exe = d / "rigid.cpp", d / "rigid"
    src.write_text(PROGRAM)
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    return exe


def test_rigid_error(program):
    r = subprocess.run([str(program)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
