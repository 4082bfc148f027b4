// Projective TSDF integration (projective_tsdf.cu:5-140) and Amanatides-Woo ray
// casting (voxel_traversal.cu:4-424) over the device-resident volume.
//
// Integration keeps the reference's per-voxel arithmetic operation for operation, but
// (a) voxel centres are computed from the index instead of read from three coordinate
// arrays, (b) everything that depends only on the frame or on the pixel a voxel lands
// in (T^-1, the in-front axis, the measured point's distance along the pixel ray and
// 1/|R lambda|) is computed once (integrate_prep) and looked up, and (c) a voxel's
// value and weight are read and written only when the voxel is updated.  The grid is
// walked one thread per (x, y) column segment with x fastest, so a warp's updates are
// 32 consecutive voxels.
#include "kf_kernels.h"
#include "kf_launch.cuh"

namespace kf {

namespace {

struct VolF32 {
    float* t;
    float* w;
    __device__ __forceinline__ void load(int i, float& tv, float& wv) const
    {
        tv = t[i];
        wv = w[i];
    }
    __device__ __forceinline__ void store(int i, float tv, float wv) const
    {
        t[i] = tv;
        w[i] = wv;
    }
};

struct VolF16 {
    __half2* p;
    __device__ __forceinline__ void load(int i, float& tv, float& wv) const
    {
        const float2 v = __half22float2(p[i]);
        tv = v.x;
        wv = v.y;
    }
    __device__ __forceinline__ void store(int i, float tv, float wv) const { p[i] = __floats2half2_rn(tv, wv); }
};

// Read-only views for the ray cast.  raw() loads a voxel without converting it, so a
// prefetched load is not waited for until decode() at its use.
struct ViewF32 {
    using Raw = float;
    const float* t;
    __device__ __forceinline__ float value(int i) const { return __ldg(t + i); }
    __device__ __forceinline__ Raw raw(int i) const { return __ldg(t + i); }
    __device__ static __forceinline__ float decode(Raw r) { return r; }
};

struct ViewF16 {
    using Raw = unsigned;  // the (value, weight) pair's bits; the value is the low half
    const __half2* p;
    __device__ __forceinline__ float value(int i) const { return __half2float(__low2half(__ldg(p + i))); }
    __device__ __forceinline__ Raw raw(int i) const { return __ldg(reinterpret_cast<const unsigned*>(p) + i); }
    __device__ static __forceinline__ float decode(Raw r)
    {
        return __half2float(__ushort_as_half((unsigned short)(r & 0xffffu)));
    }
};

// Per pixel (u, v) (1-based): the quantities of projective_tsdf.cu:39-95 that depend
// only on the pixel and the pose.  tab = (predicted_depth or NaN where the depth is
// 0, 1 / |ray direction|).  Thread 0 also stores T^-1 (cv::Mat::inv, :149) and the
// in-front axis (:57-71).
__device__ __forceinline__ void integrate_prep_at(int i, const float* __restrict__ depth, float2* __restrict__ tab,
                                                  const Camera& cam, State* st)
{
    const float* K = cam.K;
    const float* Ki = cam.Ki;
    float T[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) T[k] = st->T[k];
    if (i == 0) {
        inv4(T, st->Tinv);
        const float3 ca = mul3(Ki, make_float3(K[5], K[2], 1.f));
        const float3 cb = make_float3(2 * (Ki[0] * K[5] + Ki[1] * K[2] + Ki[2] * 1.f),
                                      2 * (Ki[3] * K[5] + Ki[4] * K[2] + Ki[5] * 1.f),
                                      2 * (Ki[6] * K[5] + Ki[7] * K[2] + Ki[8] * 1.f));
        const float3 ga = xform(T, ca), gb = xform(T, cb);
        st->axis[0] = gb.x - ga.x;
        st->axis[1] = gb.y - ga.y;
        st->axis[2] = gb.z - ga.z;
    }
    if (i >= cam.H * cam.W) return;
    const int u = i % cam.W + 1, v = i / cam.W + 1;
    const float3 lam = make_float3(Ki[0] * (float)u + Ki[1] * (float)v + Ki[2] * 1.f,
                                   Ki[3] * (float)u + Ki[4] * (float)v + Ki[5] * 1.f,
                                   Ki[6] * (float)u + Ki[7] * (float)v + Ki[8] * 1.f);
    const float3 rs = xform(T, lam);
    const float3 rd = make_float3(T[0] * 2 * lam.x + T[1] * 2 * lam.y + T[2] * 2 * lam.z + T[3],
                                  T[4] * 2 * lam.x + T[5] * 2 * lam.y + T[6] * 2 * lam.z + T[7],
                                  T[8] * 2 * lam.x + T[9] * 2 * lam.y + T[10] * 2 * lam.z + T[11]);
    const float3 dir = make_float3(rd.x - rs.x, rd.y - rs.y, rd.z - rs.z);
    const float mag = sqrtf(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    const float D = depth[i];
    const float3 pt = xform(T, make_float3(D * lam.x, D * lam.y, D * lam.z));
    const float3 rel = make_float3(pt.x - T[3], pt.y - T[7], pt.z - T[11]);
    const float dist = sqrtf(rel.x * rel.x + rel.y * rel.y + rel.z * rel.z);
    const float pd = dist / mag;
    tab[i] = make_float2(D != 0 ? pd : qnan(), 1.f / mag);
}

__global__ void __launch_bounds__(256) integrate_prep_kernel(const float* __restrict__ depth, float2* __restrict__ tab,
                                                             Camera cam, State* st)
{
    wait_for_producer();
    integrate_prep_at(blockIdx.x * blockDim.x + threadIdx.x, depth, tab, cam, st);
}

__global__ void __launch_bounds__(256) integrate_prep_batch_kernel(const SceneDev* __restrict__ scenes)
{
    wait_for_producer();
    const SceneDev& d = scenes[blockIdx.y];
    integrate_prep_at(blockIdx.x * blockDim.x + threadIdx.x, d.depth[0], d.tab, d.cam[0], d.st);
}

constexpr int kIntTx = 32, kIntTy = 8;

template <class Vol, bool FIRST>
__device__ __forceinline__ void integrate_at(const Vol& vol, const float2* __restrict__ tab,
                                             const State* __restrict__ st, const Grid& g, float fx, float fy, float cx,
                                             float cy, int H, int W, int zchunk, long long skip_from, int bx, int by,
                                             int bz)
{
    const int x = bx * kIntTx + threadIdx.x;
    const int y = by * kIntTy + threadIdx.y;
    if (x >= g.dx || y >= g.dy) return;
    const int z0 = bz * zchunk;
    const int z1 = min(z0 + zchunk, g.dz);
    float ti[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) ti[k] = st->Tinv[k];
    const float tx = st->T[3], ty = st->T[7], tz = st->T[11];
    const float ax = st->axis[0], ay = st->axis[1], az = st->axis[2];
    const float vcx = centre(x, g.sx, g.vd), vcy = centre(y, g.sy, g.vd);
    // the first two products of each row of T^-1 c and of the in-front dot product and
    // |c - t|^2 are the same along the column (left-to-right evaluation)
    const float a0 = ti[0] * vcx + ti[1] * vcy;
    const float a1 = ti[4] * vcx + ti[5] * vcy;
    const float a2 = ti[8] * vcx + ti[9] * vcy;
    const float tdx = vcx - tx, tdy = vcy - ty;
    const float f0 = ax * tdx + ay * tdy;
    const float m0 = tdx * tdx + tdy * tdy;
    {
        // Chunk cull.  The chunk's voxels lie on a segment along z.  The in-front value
        // front(z) = f0 + az (vcz - tz) and lz(z) are affine in the voxel centre vcz
        // (monotone in z), and while lz > 50 mm on the whole segment the projection
        // q(z) = (fx lx + cx lz) / lz is monotone too, so its values at the two ends bound
        // every voxel's.  The margins (1e-2 mm + 1e-5 relative on front, 1 pixel on q)
        // exceed the float error of any single voxel's evaluation by orders of magnitude,
        // so a culled chunk holds no voxel the per-voxel tests below would accept.
        float fr[2], lzv[2], qu[2], qv[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float vcz = centre(e == 0 ? z0 : z1 - 1, g.sz, g.vd);
            fr[e] = f0 + az * (vcz - tz);
            const float lx = (a0 + ti[2] * vcz) + ti[3];
            const float ly = (a1 + ti[6] * vcz) + ti[7];
            lzv[e] = (a2 + ti[10] * vcz) + ti[11];
            qu[e] = (fx * lx + cx * lzv[e]) / lzv[e];
            qv[e] = (fy * ly + cy * lzv[e]) / lzv[e];
        }
        const float fm = 1e-2f + 1e-5f * (fabsf(f0) + fabsf(fr[0]) + fabsf(fr[1]));
        bool cull = fr[0] < -fm && fr[1] < -fm;
        if (!cull && lzv[0] > 50.f && lzv[1] > 50.f) {
            const float lo = 0.5f - 1.f, hu = (float)W + 1.5f, hv = (float)H + 1.5f;
            cull = (qu[0] < lo && qu[1] < lo) || (qu[0] > hu && qu[1] > hu) || (qv[0] < lo && qv[1] < lo) ||
                   (qv[0] > hv && qv[1] > hv);
        }
        if (cull) return;
    }
    const long long rbase = ((long long)x * g.dy + y) * g.dz;
    // the reference's guard compares the thread index with the voxel count in float, so
    // the last z-fastest indices are never integrated; only the last columns get there
    const bool may_skip = rbase + z1 > skip_from;
    const int zstride = g.dx * g.dy;  // < 2^31 voxels (checked at kf_create)
    int lin = (z0 * g.dy + y) * g.dx + x;
    // a voxel projects to a pixel of the image iff q = px/pz lies in [0.5, W + 0.5) (and
    // likewise for v); q_approx = px * rcp.approx(pz) is within 2^-21 |q| of the IEEE
    // quotient, so a voxel whose q_approx is outside the range widened by that bound is
    // outside exactly and needs neither division (NaN compares false and falls through)
    const float ulo = 0.5f - 1e-3f, uhi = (float)W + 0.5f + 1e-3f * (float)W;
    const float vlo = 0.5f - 1e-3f, vhi = (float)H + 0.5f + 1e-3f * (float)H;
    for (int z = z0; z < z1; ++z, lin += zstride) {
        if (may_skip && rbase + z >= skip_from) continue;
        const float vcz = centre(z, g.sz, g.vd);
        // the reference's tests are independent rejections (all must pass), so the
        // cheapest runs first: the in-front test (:57-73) needs no projection
        const float tdz = vcz - tz;
        const float front = f0 + az * tdz;
        if (!(front > 0)) continue;
        const float lx = (a0 + ti[2] * vcz) + ti[3];
        const float ly = (a1 + ti[6] * vcz) + ti[7];
        const float lz = (a2 + ti[10] * vcz) + ti[11];
        // K (lx, ly, lz) with K's structural zeros dropped; adding a 0 product changes at
        // most the sign of a zero result, which projects to pixel 0 and is rejected
        // either way
        const float px = fx * lx + cx * lz;
        const float py = fy * ly + cy * lz;
        float r;
        asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(lz));
        const float qu = px * r, qv = py * r;
        if (qu < ulo || qu > uhi || qv < vlo || qv > vhi) continue;
        const int u = (int)roundf(px / lz);
        const int v = (int)roundf(py / lz);
        if (u < 1 || u > W || v < 1 || v > H) continue;
        const float2 e = __ldg(tab + (v - 1) * W + (u - 1));
        if (isnan(e.x)) continue;
        const float tm = sqrtf(m0 + tdz * tdz);
        const float frk = e.x - e.y * tm;
        const bool ahead = frk > 0 && frk <= g.sdf_max;
        const bool behind = frk <= 0 && frk >= g.sdf_min;
        if (!ahead && !behind) continue;
        const float f = ahead ? fminf(1.f, frk / g.trunc) : fmaxf(-1.f, frk / g.trunc);
        if (FIRST) {
            vol.store(lin, f, 1.0f);
        } else {
            float t, w;
            vol.load(lin, t, w);
            if (isnan(t)) t = 0.0f;
            if (isnan(w)) w = 0.0f;
            vol.store(lin, (w * t + 1.0f * f) / (w + 1.0f), w + 1.0f);
        }
    }
}

template <class Vol, bool FIRST>
__global__ void __launch_bounds__(kIntTx* kIntTy) integrate_kernel(Vol vol, const float2* __restrict__ tab,
                                                                   const State* __restrict__ st, Grid g, float fx,
                                                                   float fy, float cx, float cy, int H, int W,
                                                                   int zchunk, long long skip_from)
{
    wait_for_producer();
    integrate_at<Vol, FIRST>(vol, tab, st, g, fx, fy, cx, cy, H, W, zchunk, skip_from, blockIdx.x, blockIdx.y,
                             blockIdx.z);
}

__device__ __forceinline__ VolF32 scene_volume(const SceneDev& d, VolF32*) { return VolF32{d.tsdf, d.weight}; }
__device__ __forceinline__ VolF16 scene_volume(const SceneDev& d, VolF16*) { return VolF16{d.vol16}; }

// every scene's integration: blockIdx.y picks the scene, blockIdx.x its (x, y, z-chunk)
// tile; scenes with fewer tiles than the largest return early
template <class Vol, bool FIRST>
__global__ void __launch_bounds__(kIntTx* kIntTy) integrate_batch_kernel(const SceneDev* __restrict__ scenes, int zchunk)
{
    wait_for_producer();
    const SceneDev& d = scenes[blockIdx.y];
    const Grid& g = d.grid;
    const int nbx = (g.dx + kIntTx - 1) / kIntTx, nby = (g.dy + kIntTy - 1) / kIntTy, nbz = (g.dz + zchunk - 1) / zchunk;
    const int t = blockIdx.x;
    if (t >= nbx * nby * nbz) return;
    const Camera& cam = d.cam[0];
    const Vol vol = scene_volume(d, (Vol*)nullptr);
    integrate_at<Vol, FIRST>(vol, d.tab, d.st, g, cam.K[0], cam.K[4], cam.K[2], cam.K[5], cam.H, cam.W, zchunk,
                             d.skip_from, t % nbx, (t / nbx) % nby, t / (nbx * nby));
}

// Ray_Box_Intersection, voxel_traversal.cu:4-73
__device__ __forceinline__ float slab_entry(bool& inside, float3 d, float3 lo, float3 hi, float3 o)
{
    float t0, t1, ty0, ty1, tz0, tz1;
    if (d.x >= 0) {
        t0 = (lo.x - o.x) / d.x;
        t1 = (hi.x - o.x) / d.x;
    } else {
        t0 = (hi.x - o.x) / d.x;
        t1 = (lo.x - o.x) / d.x;
    }
    if (d.y >= 0) {
        ty0 = (lo.y - o.y) / d.y;
        ty1 = (hi.y - o.y) / d.y;
    } else {
        ty0 = (hi.y - o.y) / d.y;
        ty1 = (lo.y - o.y) / d.y;
    }
    if ((t0 > ty1) || (ty0 > t1)) {
        inside = false;
        return -1;
    }
    if (ty0 > t0) t0 = ty0;
    if (ty1 < t1) t1 = ty1;
    if (d.z >= 0) {
        tz0 = (lo.z - o.z) / d.z;
        tz1 = (hi.z - o.z) / d.z;
    } else {
        tz0 = (hi.z - o.z) / d.z;
        tz1 = (lo.z - o.z) / d.z;
    }
    if ((t0 > tz1) || (tz0 > t1)) {
        inside = false;
        return -1;
    }
    if (tz0 > t0) t0 = tz0;
    inside = true;
    return t0;
}

// One ray of Voxel_Traversal (voxel_traversal.cu:90-422).  The axis records XY..ZY
// start at 0, so a zero crossing met before the ray has stepped along every axis is
// not a hit (the reference leaves them uninitialised; zero is what g++ -O2 gives).
template <class View>
__device__ __forceinline__ void trace(const View& vol, float X, float Y, float D, const float* Ki, const float* T,
                                      const Grid& g, float c_flip, float4& op, float4& on, int& oh)
{
    const int L = g.dx, Wd = g.dy, Hz = g.dz;
    const float vd = g.vd;
    const float3 lo = make_float3((float)(g.sx * vd), (float)(g.sy * vd), (float)(g.sz * vd));
    const float3 hi = make_float3((float)((g.sx + L) * vd), (float)((g.sy + Wd) * vd), (float)((g.sz + Hz) * vd));
    const float3 lam = make_float3(Ki[0] * X + Ki[1] * Y + Ki[2] * 1.f, Ki[3] * X + Ki[4] * Y + Ki[5] * 1.f,
                                   Ki[6] * X + Ki[7] * Y + Ki[8] * 1.f);
    const float ln = sqrtf(lam.x * lam.x + lam.y * lam.y + lam.z * lam.z);
    // start truncated_distance before the measurement (:99-106)
    const float sc = (ln * D - g.trunc) / ln;
    const float3 sl = make_float3(sc * lam.x, sc * lam.y, sc * lam.z);
    const float3 org = make_float3(T[0] * sl.x + T[1] * sl.y + T[2] * sl.z + T[3] * 1.f,
                                   T[4] * sl.x + T[5] * sl.y + T[6] * sl.z + T[7] * 1.f,
                                   T[8] * sl.x + T[9] * sl.y + T[10] * sl.z + T[11] * 1.f);
    const float3 cam = make_float3(T[3], T[7], T[11]);
    const float3 lg = make_float3(T[0] * lam.x + T[1] * lam.y + T[2] * lam.z + T[3] * 1.f,
                                  T[4] * lam.x + T[5] * lam.y + T[6] * lam.z + T[7] * 1.f,
                                  T[8] * lam.x + T[9] * lam.y + T[10] * lam.z + T[11] * 1.f);
    const float3 dir = normalized(make_float3(lg.x - cam.x, lg.y - cam.y, lg.z - cam.z));

    bool inside = false;
    float tmin = slab_entry(inside, dir, lo, hi, org);
    if (!inside) return;
    if (tmin < 0) tmin = 0;
    const float3 s = make_float3(org.x + tmin * dir.x, org.y + tmin * dir.y, org.z + tmin * dir.z);
    const float3 box = make_float3(hi.x - lo.x, hi.y - lo.y, hi.z - lo.z);
    int ix = (int)floorf(((s.x - lo.x) / box.x) * L) + 1;
    int iy = (int)floorf(((s.y - lo.y) / box.y) * Wd) + 1;
    int iz = (int)floorf(((s.z - lo.z) / box.z) * Hz) + 1;
    int XY = 0, XZ = 0, YX = 0, YZ = 0, ZX = 0, ZY = 0;
    if (ix == L + 1) ix = ix - 1;
    if (iy == Wd + 1) iy = iy - 1;
    if (iz == Hz + 1) iz = iz - 1;
    float tvx, tvy, tvz;
    int sx, sy, sz;  // the reference steps by a float +-1; integer steps give the same indices
    if (dir.x >= 0) {
        tvx = (float)(ix) / L;
        sx = 1;
    } else {
        tvx = (float)(ix - 1) / L;
        sx = -1;
    }
    if (dir.y >= 0) {
        tvy = (float)(iy) / Wd;
        sy = 1;
    } else {
        tvy = (float)(iy - 1) / Wd;
        sy = -1;
    }
    if (dir.z >= 0) {
        tvz = (float)(iz) / Hz;
        sz = 1;
    } else {
        tvz = (float)(iz - 1) / Hz;
        sz = -1;
    }
    const float3 vmax = make_float3(lo.x + tvx * box.x, lo.y + tvy * box.y, lo.z + tvz * box.z);
    float3 tm = make_float3(tmin + ((vmax.x - s.x) / dir.x), tmin + ((vmax.y - s.y) / dir.y),
                            tmin + ((vmax.z - s.z) / dir.z));
    const float3 td = make_float3(vd / fabsf(dir.x), vd / fabsf(dir.y), vd / fabsf(dir.z));
    const int ys = L, zs = L * Wd;  // < 2^31 voxels (checked at kf_create)
    const int dlx = sx, dly = sy * ys, dlz = sz * zs;
    auto lin = [&](int a, int b, int c) -> int { return c * zs + b * ys + a; };
    int li = lin(ix - 1, iy - 1, iz - 1);

    // 0 < i < n-1 as one unsigned compare per axis
    auto inside_grid = [&](int a, int b, int c) {
        return (unsigned)(a - 1) < (unsigned)(L - 2) && (unsigned)(b - 1) < (unsigned)(Wd - 2) &&
               (unsigned)(c - 1) < (unsigned)(Hz - 2);
    };
    // The Amanatides-Woo step (:384-417) without branches: the same three comparisons
    // pick the axis; selects apply the step.
    auto pick = [](float3 t, bool& bx, bool& by, bool& bz) {
        const bool xy = t.x < t.y, xz = t.x < t.z, yz = t.y < t.z;
        bx = xy && xz;
        by = !xy && yz;
        bz = !(bx || by);
    };
    // The stepping never depends on the loaded values, only the termination does, so a
    // lead walker with the same arithmetic runs kAhead steps in front: at each position
    // it issues the voxel's load into a register ring and records, beside it, whether
    // the position is inside the loop bounds and which axis the step from it takes.  The
    // trailing walk consumes value, flag and axis in order, so it repeats neither the
    // bounds test nor the t_max comparisons.  The lead loads only voxels inside the
    // bounds.
    constexpr int kAhead = 4;
    int ax = ix, ay = iy, az = iz, ali = li;
    float3 atm = tm;
    // one Amanatides-Woo step of the lead; returns the axis (0 x, 1 y, 2 z)
    auto lead_step = [&]() -> int {
        bool bx, by, bz;
        pick(atm, bx, by, bz);
        ax += bx ? sx : 0;
        ay += by ? sy : 0;
        az += bz ? sz : 0;
        ali += bx ? dlx : (by ? dly : dlz);
        const float nx = atm.x + td.x, ny = atm.y + td.y, nz = atm.z + td.z;
        atm.x = bx ? nx : atm.x;
        atm.y = by ? ny : atm.y;
        atm.z = bz ? nz : atm.z;
        return bx ? 0 : (by ? 1 : 2);
    };
    typename View::Raw ring[kAhead];
    int code[kAhead];  // 4: inside the bounds, | axis of the step
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
        const bool in = inside_grid(ax, ay, az);
        ring[k] = in ? vol.raw(ali) : typename View::Raw(0);
        code[k] = (in ? 4 : 0) | lead_step();
    }
    float prev = 0.0f;
    float crossing = 0.f;  // the negative value met right after a positive one, or 0
    bool done = false;
    // every step moves one index one step in a fixed direction, so the walk ends within
    // L + Wd + Hz steps; the bound only makes that explicit
    for (int guard = 0; !done && guard < L + Wd + Hz + 4; guard += kAhead) {
#pragma unroll
        for (int k = 0; k < kAhead; ++k) {
            const int c = code[k];
            if (!(c & 4)) {
                done = true;
                break;
            }
            const float cur = View::decode(ring[k]);
            const bool in = inside_grid(ax, ay, az);
            ring[k] = in ? vol.raw(ali) : typename View::Raw(0);
            code[k] = (in ? 4 : 0) | lead_step();
            // the reference's four tests (:207-222) are mutually exclusive in prev
            const bool stop = prev < 0.f ? !(cur <= 0.f) : (isnan(prev) && cur < 0.f);
            if (stop) {
                done = true;
                break;
            }
            if (prev > 0.f && cur < 0.f) {
                // zero crossing: leave the walk with the state as it is and resolve it
                // below, where the warp's lanes have reconverged
                crossing = cur;
                done = true;
                break;
            }
            prev = cur;
            const int axis = c & 3;
            const bool bx = axis == 0, by = axis == 1, bz = axis == 2;
            const int ox = ix, oy = iy, oz = iz;
            XY = bx ? oy : XY;
            XZ = bx ? oz : XZ;
            YX = by ? ox : YX;
            YZ = by ? oz : YZ;
            ZX = bz ? ox : ZX;
            ZY = bz ? oy : ZY;
            ix += bx ? sx : 0;
            iy += by ? sy : 0;
            iz += bz ? sz : 0;
            li += bx ? dlx : (by ? dly : dlz);
        }
    }
    if (!(crossing < 0.f)) return;
    const float cur = crossing;
    const int xn = (ix - 1) - 1, xp = (ix - 1) + 1;
    const int yn = (iy - 1) - 1, yp = (iy - 1) + 1;
    const int zn = (iz - 1) - 1, zp = (iz - 1) + 1;
    // :233-282; recorded indices are checked against the stepped axis' extent
    if (xn >= L || xn < 0 || xp >= L || xp < 0) return;
    if ((XY - 1) >= L || (XY - 1) < 0 || (XZ - 1) >= L || (XZ - 1) < 0) return;
    if (yn >= Wd || yn < 0 || yp >= Wd || yp < 0) return;
    if ((YX - 1) >= Wd || (YX - 1) < 0 || (YZ - 1) >= Wd || (YZ - 1) < 0) return;
    if (zn >= Hz || zn < 0 || zp >= Hz || zp < 0) return;
    if ((ZX - 1) >= Hz || (ZX - 1) < 0 || (ZY - 1) >= Hz || (ZY - 1) < 0) return;
    // the recorded indices are in range for their own axes (they were loop positions),
    // so every neighbour below lies inside the grid
    const float v_xnp = vol.value(lin(xn, XY - 1, XZ - 1));
    const float v_xpp = vol.value(lin(xp, XY - 1, XZ - 1));
    const float v_ynp = vol.value(lin(YX - 1, yn, YZ - 1));
    const float v_ypp = vol.value(lin(YX - 1, yp, YZ - 1));
    const float v_znp = vol.value(lin(ZX - 1, ZY - 1, zn));
    const float v_zpp = vol.value(lin(ZX - 1, ZY - 1, zp));
    const float v_xnn = vol.value(li - 1);
    const float v_xpn = vol.value(li + 1);
    const float v_ynn = vol.value(li - ys);
    const float v_ypn = vol.value(li + ys);
    const float v_znn = vol.value(li - zs);
    const float v_zpn = vol.value(li + zs);
    if (isnan(v_xnp) || isnan(v_xpp) || isnan(v_ynp) || isnan(v_ypp) || isnan(v_znp) || isnan(v_zpp)) return;
    if (isnan(v_xnn) || isnan(v_xpn) || isnan(v_ynn) || isnan(v_ypn) || isnan(v_znn) || isnan(v_zpn)) return;
    float3 sp;
    // per-axis linear zero crossing (:318-349)
    if (dir.x > 0)
        sp.x = centre(xn, g.sx, vd) + vd * (fabsf(v_xnp) / (fabsf(v_xnp - cur)));
    else
        sp.x = centre(xp, g.sx, vd) - vd * (fabsf(v_xpp) / (fabsf(v_xpp - cur)));
    if (dir.y > 0)
        sp.y = centre(yn, g.sy, vd) + vd * (fabsf(v_ynp) / (fabsf(v_ynp - cur)));
    else
        sp.y = centre(yp, g.sy, vd) - vd * (fabsf(v_ypp) / (fabsf(v_ypp - cur)));
    if (dir.z > 0)
        sp.z = centre(zn, g.sz, vd) + vd * (fabsf(v_znp) / (fabsf(v_znp - cur)));
    else
        sp.z = centre(zp, g.sz, vd) - vd * (fabsf(v_zpp) / (fabsf(v_zpp - cur)));
    const float3 nr = make_float3((v_xpn - v_xnn) / 2.0f, (v_ypn - v_ynn) / 2.0f, (v_zpn - v_znn) / 2.0f);
    const float3 va = normalized(make_float3(cam.x - sp.x, cam.y - sp.y, cam.z - sp.z));
    float3 vb = normalized(nr);
    const float ct = va.x * vb.x + va.y * vb.y + va.z * vb.z;
    if (ct < c_flip) vb = make_float3(-vb.x, -vb.y, -vb.z);
    op = make_float4(sp.x, sp.y, sp.z, 0.f);
    on = make_float4(vb.x, vb.y, vb.z, 0.f);
    oh = ((ix - 1) * Wd + (iy - 1)) * Hz + (iz - 1);
}

// Persistent: each warp takes 8x4-pixel tiles (one ray per lane) from a counter until
// none are left, so the spatially clustered long walks do not leave a tail of idle SMs.
// Tiles are numbered row-major, so consecutive tiles are neighbours in the image.
constexpr int kRayBlock = 256;

template <class View>
__global__ void __launch_bounds__(kRayBlock, 4) raycast_kernel(View vol, const float* __restrict__ depth,
                                                            float4* __restrict__ pv, float4* __restrict__ pn,
                                                            int32_t* __restrict__ hit, Camera cam, Grid g,
                                                            const State* __restrict__ st, unsigned* tile_counter)
{
    wait_for_producer();
    const int lane = threadIdx.x & 31;
    const int tiles_x = (cam.W + 7) / 8, ntiles = tiles_x * ((cam.H + 3) / 4);
    float T[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) T[k] = st->T[k];
    const float c_flip = st->c_flip;
    for (;;) {
        unsigned tile = 0;
        if (lane == 0) tile = atomicAdd(tile_counter, 1u);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= (unsigned)ntiles) {
            // the last warp out resets both counters for the next launch
            if (lane == 0) {
                const unsigned warps = gridDim.x * (blockDim.x / 32);
                if (atomicAdd(tile_counter + 1, 1u) == warps - 1) {
                    tile_counter[0] = 0u;
                    tile_counter[1] = 0u;
                }
            }
            return;
        }
        const int px = (int)(tile % tiles_x) * 8 + (lane & 7);
        const int py = (int)(tile / tiles_x) * 4 + (lane >> 3);
        if (px >= cam.W || py >= cam.H) continue;
        const int i = py * cam.W + px;
        float4 op = make_float4(0.f, 0.f, 0.f, 0.f), on = op;
        int oh = -1;
        const float D = depth[i];
        if (D != 0) trace(vol, (float)px + 1.0f, (float)py + 1.0f, D, cam.Ki, T, g, c_flip, op, on, oh);
        pv[i] = op;
        pn[i] = on;
        if (hit) hit[i] = oh;
    }
}

__device__ __forceinline__ ViewF32 scene_view(const SceneDev& d, ViewF32*) { return ViewF32{d.tsdf}; }
__device__ __forceinline__ ViewF16 scene_view(const SceneDev& d, ViewF16*) { return ViewF16{d.vol16}; }

// Every scene's ray cast in one persistent launch: warps take TW x (32/TW)-pixel tiles
// from one counter over all scenes' tiles (scene s owns tiles [tile_start[shape],
// tile_start[shape] of s + 1)), so uneven scenes share the SMs without a tail per scene.
template <class View, int TW, int SHAPE>
__global__ void __launch_bounds__(kRayBlock, 4) raycast_batch_kernel(const SceneDev* __restrict__ scenes, int n_scenes,
                                                                  unsigned total_tiles, unsigned* tile_counter)
{
    wait_for_producer();
    constexpr int TH = 32 / TW;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned tile = 0;
        if (lane == 0) tile = atomicAdd(tile_counter, 1u);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= total_tiles) {
            if (lane == 0) {
                const unsigned warps = gridDim.x * (blockDim.x / 32);
                if (atomicAdd(tile_counter + 1, 1u) == warps - 1) {
                    tile_counter[0] = 0u;
                    tile_counter[1] = 0u;
                }
            }
            return;
        }
        int s = 0;
        while (s + 1 < n_scenes && tile >= (unsigned)scenes[s + 1].tile_start[SHAPE]) ++s;
        const SceneDev& d = scenes[s];
        const Camera& cam = d.cam[0];
        const unsigned t = tile - (unsigned)d.tile_start[SHAPE];
        const int tiles_x = (cam.W + TW - 1) / TW;
        const int px = (int)(t % tiles_x) * TW + (lane % TW);
        const int py = (int)(t / tiles_x) * TH + lane / TW;
        if (px >= cam.W || py >= cam.H) continue;
        float T[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) T[k] = d.st->T[k];
        const int i = py * cam.W + px;
        float4 op = make_float4(0.f, 0.f, 0.f, 0.f), on = op;
        int oh = -1;
        const float D = d.depth[0][i];
        if (D != 0)
            trace(scene_view(d, (View*)nullptr), (float)px + 1.0f, (float)py + 1.0f, D, cam.Ki, T, d.grid,
                  d.st->c_flip, op, on, oh);
        d.pv[0][i] = op;
        d.pn[0][i] = on;
        if (d.hit) d.hit[i] = oh;
    }
}

}  // namespace

int raycast_blocks()
{
    static int blocks[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152 * 4;
    if (!blocks[dev]) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, raycast_kernel<ViewF32>, kRayBlock, 0);
        blocks[dev] = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 4);
    }
    return blocks[dev];
}

void launch_integrate_prep(const float* depth, float2* tab, const Camera& cam, State* st, cudaStream_t s)
{
    const int n = cam.H * cam.W;
    launch_pdl(integrate_prep_kernel, dim3((n + 255) / 256), dim3(256), 0, s, depth, tab, cam, st);
}

namespace {
constexpr int kZChunk = 16;

template <class Vol>
void integrate_launch(Vol vol, const float2* tab, const State* st, const Grid& g, const Camera& cam,
                      long long skip_from, bool first, cudaStream_t s)
{
    dim3 block(kIntTx, kIntTy);
    dim3 grid((g.dx + kIntTx - 1) / kIntTx, (g.dy + kIntTy - 1) / kIntTy, (g.dz + kZChunk - 1) / kZChunk);
    const float fx = cam.K[0], fy = cam.K[4], cx = cam.K[2], cy = cam.K[5];
    if (first)
        launch_pdl(integrate_kernel<Vol, true>, grid, block, 0, s, vol, tab, st, g, fx, fy, cx, cy, cam.H, cam.W,
                   kZChunk, skip_from);
    else
        launch_pdl(integrate_kernel<Vol, false>, grid, block, 0, s, vol, tab, st, g, fx, fy, cx, cy, cam.H, cam.W,
                   kZChunk, skip_from);
}
}  // namespace

void launch_integrate_f32(float* tsdf, float* weight, const float2* tab, const State* st, const Grid& g,
                          const Camera& cam, long long skip_from, bool first, cudaStream_t s)
{
    integrate_launch(VolF32{tsdf, weight}, tab, st, g, cam, skip_from, first, s);
}

void launch_integrate_f16(__half2* vol, const float2* tab, const State* st, const Grid& g, const Camera& cam,
                          long long skip_from, bool first, cudaStream_t s)
{
    integrate_launch(VolF16{vol}, tab, st, g, cam, skip_from, first, s);
}

void launch_raycast_f32(const float* tsdf, const float* depth, float4* pv, float4* pn, int32_t* hit,
                        const Camera& cam, const Grid& g, const State* st, unsigned* tile_counter, cudaStream_t s)
{
    launch_pdl(raycast_kernel<ViewF32>, dim3(raycast_blocks()), dim3(kRayBlock), 0, s, ViewF32{tsdf}, depth, pv, pn,
               hit, cam, g, st, tile_counter);
}

void launch_raycast_f16(const __half2* vol, const float* depth, float4* pv, float4* pn, int32_t* hit,
                        const Camera& cam, const Grid& g, const State* st, unsigned* tile_counter, cudaStream_t s)
{
    launch_pdl(raycast_kernel<ViewF16>, dim3(raycast_blocks()), dim3(kRayBlock), 0, s, ViewF16{vol}, depth, pv, pn,
               hit, cam, g, st, tile_counter);
}

void launch_integrate_batch(const SceneDev* scenes, int n_scenes, int max_pixels, int max_tiles, int zchunk, bool f16,
                            bool first, cudaStream_t s)
{
    launch_pdl(integrate_prep_batch_kernel, dim3((max_pixels + 255) / 256, n_scenes), dim3(256), 0, s, scenes);
    const dim3 grid(max_tiles, n_scenes), block(kIntTx, kIntTy);
    if (f16) {
        if (first)
            launch_pdl(integrate_batch_kernel<VolF16, true>, grid, block, 0, s, scenes, zchunk);
        else
            launch_pdl(integrate_batch_kernel<VolF16, false>, grid, block, 0, s, scenes, zchunk);
    } else {
        if (first)
            launch_pdl(integrate_batch_kernel<VolF32, true>, grid, block, 0, s, scenes, zchunk);
        else
            launch_pdl(integrate_batch_kernel<VolF32, false>, grid, block, 0, s, scenes, zchunk);
    }
}

int integrate_tiles(const Grid& g, int zchunk)
{
    return ((g.dx + kIntTx - 1) / kIntTx) * ((g.dy + kIntTy - 1) / kIntTy) * ((g.dz + zchunk - 1) / zchunk);
}

int raycast_tiles(int H, int W, int shape)
{
    const int tw = shape == 1 ? 16 : (shape == 2 ? 4 : 8), th = 32 / tw;
    return ((W + tw - 1) / tw) * ((H + th - 1) / th);
}

void launch_raycast_batch(const SceneDev* scenes, int n_scenes, unsigned total_tiles, bool f16, int shape,
                          int blocks, unsigned* tile_counter, cudaStream_t s)
{
    const dim3 grid(blocks), block(kRayBlock);
#define KF_RAY_BATCH(VIEW, TW, SH) \
    launch_pdl(raycast_batch_kernel<VIEW, TW, SH>, grid, block, 0, s, scenes, n_scenes, total_tiles, tile_counter)
    if (f16) {
        if (shape == 1)
            KF_RAY_BATCH(ViewF16, 16, 1);
        else if (shape == 2)
            KF_RAY_BATCH(ViewF16, 4, 2);
        else
            KF_RAY_BATCH(ViewF16, 8, 0);
    } else {
        if (shape == 1)
            KF_RAY_BATCH(ViewF32, 16, 1);
        else if (shape == 2)
            KF_RAY_BATCH(ViewF32, 4, 2);
        else
            KF_RAY_BATCH(ViewF32, 8, 0);
    }
#undef KF_RAY_BATCH
}

}  // namespace kf
