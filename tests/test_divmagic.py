"""The ray cast decodes linear voxel indices with kf_divmagic.h's multiply-high division
(Granlund-Montgomery, N = 31).  Its host form is compiled here with g++ and checked
against the exact quotient for every divisor from 2 to 4096 (the grid sides are 3 to
4096) and larger ones, at dividends around every multiple of the divisor near the ends
of the range and at random ones below 2^31."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "kinect_fusion_slam_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include "kf_divmagic.h"

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint32_t next31()
{
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (uint32_t)(state >> 33);
}

static int check(uint32_t d, int32_t n, kf::DivMagic q)
{
    if (n < 0) return 0;
    if (kf::div_by(n, q) != n / (int32_t)d) {
        std::printf("d=%u n=%d got %d want %d\n", d, n, kf::div_by(n, q), n / (int32_t)d);
        return 1;
    }
    return 0;
}

int main()
{
    int bad = 0;
    uint32_t ds[4200];
    int nd = 0;
    for (uint32_t d = 2; d <= 4096; ++d) ds[nd++] = d;
    const uint32_t big[] = {4097, 65535, 65536, 65537, 1000003, 46341, 2147483647u, 1073741825u, 1073741824u};
    for (uint32_t d : big) ds[nd++] = d;
    for (int k = 0; k < nd; ++k) {
        const uint32_t d = ds[k];
        const kf::DivMagic q = kf::div_magic(d);
        if (q.s < 0) { std::printf("d=%u shift %d\n", d, q.s); return 1; }
        const int64_t top = 2147483647;
        // around the first and the last multiples of d, and at every multiple for small n
        for (int64_t j = 0; j <= 2100; ++j)
            for (int r = -1; r <= 1; ++r) {
                bad += check(d, (int32_t)(j * d + r), q);
                const int64_t hi = (top / d - j) * (int64_t)d + r;
                if (hi >= 0 && hi <= top) bad += check(d, (int32_t)hi, q);
            }
        for (int t = 0; t < 20000; ++t) bad += check(d, (int32_t)next31(), q);
        bad += check(d, (int32_t)top, q);
        if (bad) return 1;
    }
    std::printf("ok %d divisors\n", nd);
    return 0;
}
"""


def test_div_magic_is_exact(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "divmagic.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "divmagic"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")
