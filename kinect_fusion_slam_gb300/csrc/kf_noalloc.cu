// kf_icp_associate_noalloc: the ICP association and normal-equation reduction on
// caller-owned device buffers, with no device allocation.
//
// Some callers cannot allocate device memory at the point where they want this
// operator: a real-time loop that must not stall on cudaMalloc (which can synchronise
// the device and take driver locks), or a host application that hands out all GPU
// memory from its own pre-reserved pool.  For them the scratch this reduction needs
// (one 28-float partial per 64-pixel group, a group list, a completion counter and the
// two 4x4 transforms) lives in one file-scope static device array sized for images
// of up to kNoAllocMaxPixels pixels.  Every GPU that loads this library holds that
// array (about 0.55 MB) until the process exits.
//
// Host code cannot use the array's name as a device address (on the host it is a
// stand-in symbol), so the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current and caches it.  That first call
// should therefore come before any stream capture.  All calls share the array and it
// keeps the last call's contents: each call re-initialises the parts that must start
// from zero, and calls that overlap on the GPU (different streams at once) race on it.
#include <mutex>

#include "kinfu_gb300.h"
#include "kf_kernels.h"

namespace {

using kf::kIcpVals;

constexpr int kNoAllocMaxPixels = 640 * 480;
constexpr int kNoAllocMaxGroups = (kNoAllocMaxPixels + 63) / 64;
constexpr int kMaxDevices = 64;

constexpr size_t round256(size_t n) { return (n + 255) / 256 * 256; }
constexpr size_t kStateOff = 0;
constexpr size_t kMatsOff = kStateOff + round256(sizeof(kf::State));
constexpr size_t kPartialsOff = kMatsOff + round256(32 * sizeof(float));
constexpr size_t kPartialFloats = (size_t)kNoAllocMaxGroups * kIcpVals;
constexpr size_t kListOff = kPartialsOff + round256(kPartialFloats * sizeof(float));
constexpr size_t kScratchBytes = kListOff + round256((size_t)kNoAllocMaxGroups * sizeof(int));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct Mats {
    float F[16];
    float T[16];
};

// writes the call's transforms into the scratch and zeroes the completion counter and
// the error flag (the reduction's bounded waits run at their default limit)
__global__ void noalloc_prepare_kernel(Mats m)
{
    float* mats = reinterpret_cast<float*>(g_noalloc_scratch + kMatsOff);
    if (threadIdx.x < 16) {
        mats[threadIdx.x] = m.F[threadIdx.x];
        mats[16 + threadIdx.x] = m.T[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        kf::State* st = reinterpret_cast<kf::State*>(g_noalloc_scratch + kStateOff);
        st->ticket = 0u;
        st->error = 0;
        st->wait_limit = kf::kDefaultWaitLimit;
    }
}

std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {};

// device address of the scratch array on the current device (looked up once per device)
cudaError_t scratch_base(unsigned char** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_base[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_base[dev] = static_cast<unsigned char*>(p);
        kf::icp_prepare(480, 640);  // shared-memory limit of the reduce pass, sized for the largest image
    }
    *out = g_base[dev];
    return cudaSuccess;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" kf_status kf_icp_associate_noalloc(int height, int width, const float K[9], const float F[16],
                                              const float T[16], const float* vmap, const float* nmap,
                                              const float* pred_v, const float* pred_n, float dist_mm,
                                              float angle_deg, float* sums28, int32_t* pair, void* stream)
{
    if (height <= 0 || width <= 0 || !K || !F || !T || !vmap || !nmap || !pred_v || !pred_n || !sums28)
        return KF_ERR_INVALID_ARGUMENT;
    if ((long long)height * width > kNoAllocMaxPixels) return KF_ERR_UNSUPPORTED;
    if (!aligned16(vmap) || !aligned16(nmap) || !aligned16(pred_v) || !aligned16(pred_n))
        return KF_ERR_INVALID_ARGUMENT;
    if (!(dist_mm >= 0.f) || !(angle_deg >= 0.f)) return KF_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (s) {
        // the scratch address below is the current device's: the stream must be on it
        int cur = 0, sdev = 0;
        if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(s, &sdev) != cudaSuccess) return KF_ERR_CUDA;
        if (sdev != cur) return KF_ERR_INVALID_ARGUMENT;
    }
    unsigned char* base = nullptr;
    if (scratch_base(&base) != cudaSuccess) return KF_ERR_CUDA;

    kf::Camera cam{};
    cam.H = height;
    cam.W = width;
    for (int k = 0; k < 9; ++k) cam.K[k] = K[k];
    kf::inv3(cam.K, cam.Ki);
    // the reference order, no fail-mode or precision choice involved in association
    const kf::IcpParams prm{dist_mm, angle_deg, 0, 0, 1};
    Mats m;
    for (int k = 0; k < 16; ++k) {
        m.F[k] = F[k];
        m.T[k] = T[k];
    }
    noalloc_prepare_kernel<<<1, 32, 0, s>>>(m);
    const float* mats = reinterpret_cast<const float*>(base + kMatsOff);
    kf::launch_icp_associate(reinterpret_cast<const float4*>(vmap), reinterpret_cast<const float4*>(nmap),
                             reinterpret_cast<const float4*>(pred_v), reinterpret_cast<const float4*>(pred_n), cam,
                             prm, mats, mats + 16, reinterpret_cast<kf::State*>(base + kStateOff),
                             reinterpret_cast<float*>(base + kPartialsOff), reinterpret_cast<int*>(base + kListOff),
                             nullptr, sums28, pair, s);
    return cudaGetLastError() == cudaSuccess ? KF_OK : KF_ERR_CUDA;
}
