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
#include "kf_rigid.h"

namespace kf {

namespace {

struct VolF32 {
    static constexpr bool kLean = false;  // the reference's arithmetic, operation for operation
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
    // the FP16 form's integration arithmetic (integrate_at): the voxel's pixel as in the
    // reference (IEEE quotients), its distance and value by approximate square root and
    // reciprocals, which the 11-bit storage cannot tell from the IEEE operations
    static constexpr bool kLean = true;
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
    // below kNegativeKeys exactly for a value < 0 (not -0, not NaN): bits in
    // [0x80000001, 0xff800000]
    __device__ static __forceinline__ unsigned negative_key(Raw r) { return __float_as_uint(r) - 0x80000001u; }
    static constexpr unsigned kNegativeKeys = 0x7f800000u;
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
    // below kNegativeKeys exactly for a value < 0 (not -0, not NaN): the value's bits in
    // [0x8001, 0xfc00], moved to the top half (the weight's bits drop out)
    __device__ static __forceinline__ unsigned negative_key(Raw r) { return (r << 16) - 0x80010000u; }
    static constexpr unsigned kNegativeKeys = 0x7c000000u;
};

// Per pixel (u, v) (1-based): the quantities of projective_tsdf.cu:39-95 that depend
// only on the pixel and the pose.  tab = (predicted_depth or NaN where the depth is
// 0, 1 / |ray direction|).  Thread 0 also stores the in-front axis (:57-71); the warp
// of tile 0 stores T^-1 (cv::Mat::inv, :149; integrate_prep_tile).
__device__ __forceinline__ void integrate_prep_at(int i, const float* __restrict__ depth, float2* __restrict__ tab,
                                                  const Camera& cam, State* st)
{
    const float* K = cam.K;
    const float* Ki = cam.Ki;
    float T[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) T[k] = st->T[k];
    if (i == 0) {
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

// Per 8x8-pixel tile of the depth image: (min, max) of its nonzero |depth|, (+inf, -inf)
// where it has none.  The table's distance entry is |D| times a factor within rounding
// of 1 (the norm of D times the ray over the ray's norm), so these bound the entries
// integration would read there.  Stored after the table's H*W entries.
constexpr int kBoundTile = 8;

__device__ __forceinline__ int bound_tiles_x(int W) { return (W + kBoundTile - 1) / kBoundTile; }

// one warp per tile, two pixels per lane: the table entries of the tile's pixels and the
// tile's depth bounds
__device__ __forceinline__ void integrate_prep_tile(int tile, int lane, const float* __restrict__ depth,
                                                    float2* __restrict__ tab, const Camera& cam, State* st)
{
    const int H = cam.H, W = cam.W;
    const int ntx = bound_tiles_x(W);
    const int x0 = (tile % ntx) * kBoundTile, y0 = (tile / ntx) * kBoundTile;
    if (tile == 0) {
        // T^-1 for integration, and the pose it inverts (the next frame's ICP reuses
        // the inverse while the pose is unchanged); an empty mark list
        inv4_warp(st->T, st->Tinv);
        if (lane < 16) st->Tinv_src[lane] = st->T[lane];
        if (lane == 0) {
            st->mark_count = 0u;
            st->mark_near = 0u;
            st->mark_all = 0u;
        }
    }
    float lo = INFINITY, hi = -INFINITY;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int x = x0 + (lane & 7), y = y0 + (lane >> 3) + 4 * h;
        if (x < W && y < H) {
            const int i = y * W + x;
            integrate_prep_at(i, depth, tab, cam, st);
            const float d = fabsf(depth[i]);
            if (d != 0.f) {
                lo = fminf(lo, d);
                hi = fmaxf(hi, d);
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    }
    if (lane == 0) tab[H * W + tile] = make_float2(lo, hi);
}

__global__ void __launch_bounds__(256) integrate_prep_kernel(const float* __restrict__ depth, float2* __restrict__ tab,
                                                             Camera cam, State* st)
{
    wait_for_producer();
    // integration may be scheduled now; it waits for this kernel before reading the table
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int tiles = bound_tiles_x(cam.W) * ((cam.H + kBoundTile - 1) / kBoundTile);
    const int tile = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (tile < tiles) integrate_prep_tile(tile, threadIdx.x & 31, depth, tab, cam, st);
}

__global__ void __launch_bounds__(256) integrate_prep_batch_kernel(const SceneDev* __restrict__ scenes)
{
    wait_for_producer();
    const SceneDev& d = scenes[blockIdx.y];
    const Camera& cam = d.cam[0];
    const int tiles = bound_tiles_x(cam.W) * ((cam.H + kBoundTile - 1) / kBoundTile);
    for (int tile = blockIdx.x * 8 + (threadIdx.x >> 5); tile < tiles; tile += gridDim.x * 8)
        integrate_prep_tile(tile, threadIdx.x & 31, d.depth[0], d.tab, cam, d.st);
}

// Integration proceeds in boxes of kIntTx x kIntTy voxel columns by zchunk voxels along
// z, a block of kIntTx x kIntTy threads per box, one thread per column segment.  A single
// scene's boxes are chosen from the depth tiles' side (integrate_mark_kernel: the boxes
// a tile's pixels can update are marked, then listed); a batch of scenes decides each
// box by its corners and its footprint's depth bounds (box_live).  Within a box every
// voxel runs the reference's tests.  (A further cull of each thread's segment by the
// corner tests cost more than the voxels it removed: 48.9 -> 44.7 us per c1 frame
// without it.)
constexpr int kIntTx = 32, kIntTy = 8;
constexpr int kZB = 4;  // voxels of a column segment whose loads are issued together (batched scenes)

// The frame's constants of integration beside the pose (which the kernels read from
// State).
struct IntegrateParams {
    float fx, fy, cx, cy;
    int H, W;
    int zchunk;
    long long skip_from;
    float depth_eps;  // relative depth margin of the depth-band cull (depth_band_eps)
    float lam_max;    // largest |K^-1 (u, v, 1)| over the image
};

__device__ __forceinline__ IntegrateParams scene_params(const SceneDev& d, int zchunk)
{
    const Camera& c = d.cam[0];
    return IntegrateParams{c.K[0], c.K[4], c.K[2], c.K[5], c.H, c.W, zchunk, d.skip_from, d.depth_eps, d.lam_max};
}

// Bounds of what integration computes over a set of voxel centres.  Every quantity the
// per-voxel tests use is affine in the centre (the in-front value, the camera-frame
// coordinates) or, while the camera depth lz stays positive, a ratio of affine
// functions (the projection q = (f l + c lz) / lz), so over a box of centres (or a
// segment) their extremes are attained at its corners (ends): for a centre that is a
// convex combination of corners, f l + c lz - q_k lz < 0 at every corner implies it for
// the centre.  The magnitude sums bound the float rounding of each evaluation.
struct Extent {
    float front, fmag;     // largest in-front value; largest sum of its terms' magnitudes
    float lz_lo, lz_hi;    // camera depth range
    float qu_lo, qu_hi;    // projection range (meaningful while lz_lo > 0)
    float qv_lo, qv_hi;
    float lmag;            // largest magnitude sum of a camera-frame coordinate's terms
};

__device__ __forceinline__ Extent corner_extent(const float* ti, float tx, float ty, float tz, float ax, float ay,
                                                float az, float vcx, float vcy, float vcz, const IntegrateParams& p)
{
    Extent e;
    const float tdx = vcx - tx, tdy = vcy - ty, tdz = vcz - tz;
    e.front = (ax * tdx + ay * tdy) + az * tdz;
    e.fmag = fabsf(ax * tdx) + fabsf(ay * tdy) + fabsf(az * tdz);
    const float lx = (ti[0] * vcx + ti[1] * vcy) + ti[2] * vcz + ti[3];
    const float ly = (ti[4] * vcx + ti[5] * vcy) + ti[6] * vcz + ti[7];
    const float lz = (ti[8] * vcx + ti[9] * vcy) + ti[10] * vcz + ti[11];
    e.lz_lo = e.lz_hi = lz;
    e.qu_lo = e.qu_hi = (p.fx * lx + p.cx * lz) / lz;
    e.qv_lo = e.qv_hi = (p.fy * ly + p.cy * lz) / lz;
    float m = 0.f;
#pragma unroll
    for (int r = 0; r < 3; ++r)
        m = fmaxf(m, fabsf(ti[4 * r] * vcx) + fabsf(ti[4 * r + 1] * vcy) + fabsf(ti[4 * r + 2] * vcz) +
                         fabsf(ti[4 * r + 3]));
    e.lmag = m;
    return e;
}

__device__ __forceinline__ void merge_extent(Extent& a, const Extent& b)
{
    a.front = fmaxf(a.front, b.front);
    a.fmag = fmaxf(a.fmag, b.fmag);
    a.lz_lo = fminf(a.lz_lo, b.lz_lo);
    a.lz_hi = fmaxf(a.lz_hi, b.lz_hi);
    a.qu_lo = fminf(a.qu_lo, b.qu_lo);
    a.qu_hi = fmaxf(a.qu_hi, b.qu_hi);
    a.qv_lo = fminf(a.qv_lo, b.qv_lo);
    a.qv_hi = fmaxf(a.qv_hi, b.qv_hi);
    a.lmag = fmaxf(a.lmag, b.lmag);
}

__device__ __forceinline__ Extent shfl_xor_extent(const Extent& e, int off)
{
    Extent o;
    o.front = __shfl_xor_sync(0xffffffffu, e.front, off);
    o.fmag = __shfl_xor_sync(0xffffffffu, e.fmag, off);
    o.lz_lo = __shfl_xor_sync(0xffffffffu, e.lz_lo, off);
    o.lz_hi = __shfl_xor_sync(0xffffffffu, e.lz_hi, off);
    o.qu_lo = __shfl_xor_sync(0xffffffffu, e.qu_lo, off);
    o.qu_hi = __shfl_xor_sync(0xffffffffu, e.qu_hi, off);
    o.qv_lo = __shfl_xor_sync(0xffffffffu, e.qv_lo, off);
    o.qv_hi = __shfl_xor_sync(0xffffffffu, e.qv_hi, off);
    o.lmag = __shfl_xor_sync(0xffffffffu, e.lmag, off);
    return o;
}

// Pixel footprint of an extent that survived the frustum test: the image rows and
// columns (0-based) its centres can round to, as 8x8-tile ranges.
struct Footprint {
    int tx0, tx1, ty0, ty1;
    float lz_lo, lz_hi;  // widened by the evaluation error
};

// 0: some centre may be updated and the footprint is not known (keep); 1: no centre can
// be updated (cull); 2: the depth-band test over footprint fp decides.
//
// Margins.  A voxel's own evaluation and a corner's differ from the exact affine values
// by a few roundings of their partial sums: err_l = 2^-20 lmag bounds both for the
// camera coordinates (5 roundings of at most 2^-24 lmag each, twice), and
// 1e-2 + 1e-5 fmag for the in-front value.  A voxel is kept by the projection test iff
// its rounded q lies in [0.5, W + 0.5); a q bound moves by at most
// (f + |c| + |q|) err_l / lz + 2^-20 |q| when the coordinates move by err_l, and one
// more pixel is added on top.
__device__ __forceinline__ int extent_cull(const Extent& e, const IntegrateParams& p, Footprint& fp)
{
    const float fm = 1e-2f + 1e-5f * e.fmag;
    if (e.front < -fm) return 1;
    const float err_l = e.lmag * 0x1p-20f;
    const float lz_lo = e.lz_lo - err_l;
    if (!(lz_lo > 50.f)) return 0;
    const float qabs = fmaxf(fmaxf(fabsf(e.qu_lo), fabsf(e.qu_hi)), fmaxf(fabsf(e.qv_lo), fabsf(e.qv_hi)));
    const float mq = 1.f + (fmaxf(p.fx, p.fy) + fmaxf(fabsf(p.cx), fabsf(p.cy)) + qabs) * err_l / lz_lo +
                     qabs * 0x1p-20f;
    if (e.qu_hi < 0.5f - mq || e.qu_lo >= (float)p.W + 0.5f + mq || e.qv_hi < 0.5f - mq ||
        e.qv_lo >= (float)p.H + 0.5f + mq)
        return 1;
    // column u - 1 of u = round(q) for q in [qu_lo - mq, qu_hi + mq], clamped to the image
    const float W1 = (float)(p.W - 1), H1 = (float)(p.H - 1);
    const int c0 = (int)fminf(fmaxf(floorf(e.qu_lo - mq) - 1.f, 0.f), W1);
    const int c1 = (int)fminf(fmaxf(floorf(e.qu_hi + mq), 0.f), W1);
    const int r0 = (int)fminf(fmaxf(floorf(e.qv_lo - mq) - 1.f, 0.f), H1);
    const int r1 = (int)fminf(fmaxf(floorf(e.qv_hi + mq), 0.f), H1);
    fp.tx0 = c0 / kBoundTile;
    fp.tx1 = c1 / kBoundTile;
    fp.ty0 = r0 / kBoundTile;
    fp.ty1 = r1 / kBoundTile;
    fp.lz_lo = lz_lo;
    fp.lz_hi = e.lz_hi + err_l;
    return 2;
}

// Depth-band test.  A voxel is updated only if frk = D' - tm / m lies in [sdf_min,
// sdf_max] (widened to contain 0), D' being the table's distance for its pixel and
// tm / m the voxel's distance from the camera over the pixel ray's norm.  With the pixel
// centre within half a pixel of the voxel's projection, tm / m is lz times a factor
// within depth_eps of 1.  The table's entries are computed from the pose: D' is |D| to
// within a relative eps_t plus an absolute 2^-19 |t| (rounding against the translation
// t), and m to within eps_t.  With dmin, dmax the tile bounds of |D| over the footprint,
// no voxel is updated if all of them are more than the band in front of every depth or
// behind it, with another millimetre for the rounding of frk itself.
__device__ __forceinline__ bool band_culled(const Footprint& fp, float dmin, float dmax, const IntegrateParams& p,
                                            const Grid& g, const State* __restrict__ st)
{
    const float tmax = fmaxf(fmaxf(fabsf(st->T[3]), fabsf(st->T[7])), fabsf(st->T[11]));
    const float eps_t = 0x1p-18f * (tmax + 4.f * p.lam_max + 1.f);
    const float abs_t = 0x1p-19f * tmax + 1.f;
    const float hi_band = fmaxf(g.sdf_max, 0.f), lo_band = fminf(g.sdf_min, 0.f);
    // a rotation block up to kRigidTol off orthonormal scales tm / m against lz by at most
    // 1 +- 2 kRigidTol (box_live keeps every box for a pose further off)
    const float rig = 4.f * kRigidTol;
    const bool all_ahead = fp.lz_hi * (1.f + p.depth_eps) * (1.f + eps_t) * (1.f + rig) + abs_t <
                           dmin * (1.f - eps_t) - hi_band - abs_t;
    const bool all_behind = fp.lz_lo * (1.f - p.depth_eps) * (1.f - eps_t) * (1.f - rig) - abs_t >
                            dmax * (1.f + eps_t) - lo_band + abs_t;
    return all_ahead || all_behind;
}

__device__ __forceinline__ void load_pose(const State* __restrict__ st, float* ti, float& tx, float& ty, float& tz,
                                          float& ax, float& ay, float& az)
{
#pragma unroll
    for (int k = 0; k < 12; ++k) ti[k] = st->Tinv[k];
    tx = st->T[3];
    ty = st->T[7];
    tz = st->T[11];
    ax = st->axis[0];
    ay = st->axis[1];
    az = st->axis[2];
}

// Box cull, run by one warp for its block's box of kIntTx x kIntTy columns x zchunk
// voxels: lanes 0..7 (and their copies in each group of 8) evaluate the box's eight
// corner centres, the warp merges them, and all lanes read the footprint's tile bounds.
// False if no voxel of the box can be updated.
__device__ __forceinline__ bool box_live(int bx, int by, int bz, int lane, const Grid& g,
                                         const State* __restrict__ st, const float2* __restrict__ bounds,
                                         const IntegrateParams& p)
{
    // the cull's margins hold for a rotation within kRigidTol of orthonormal; a pose
    // further off keeps every box (the same decision in every lane)
    {
        float T[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) T[k] = st->T[k];
        if (rigid_error(T) > kRigidTol) return true;
    }
    float ti[12], tx, ty, tz, ax, ay, az;
    load_pose(st, ti, tx, ty, tz, ax, ay, az);
    const int c = lane & 7;
    const int ix = (c & 1) ? min(g.dx, bx * kIntTx + kIntTx) - 1 : bx * kIntTx;
    const int iy = (c & 2) ? min(g.dy, by * kIntTy + kIntTy) - 1 : by * kIntTy;
    const int iz = (c & 4) ? min(g.dz, bz * p.zchunk + p.zchunk) - 1 : bz * p.zchunk;
    Extent e = corner_extent(ti, tx, ty, tz, ax, ay, az, centre(ix, g.sx, g.vd), centre(iy, g.sy, g.vd),
                             centre(iz, g.sz, g.vd), p);
#pragma unroll
    for (int off = 1; off < 8; off <<= 1) merge_extent(e, shfl_xor_extent(e, off));
    Footprint fp;
    const int r = extent_cull(e, p, fp);  // the same in every lane
    if (r != 2) return r == 0;
    const int ntx = bound_tiles_x(p.W), w = fp.tx1 - fp.tx0 + 1;
    const int n = w * (fp.ty1 - fp.ty0 + 1);
    float dmin = INFINITY, dmax = -INFINITY;
    for (int k = lane; k < n; k += 32) {
        const float2 b = __ldg(bounds + (fp.ty0 + k / w) * ntx + fp.tx0 + k % w);
        dmin = fminf(dmin, b.x);
        dmax = fmaxf(dmax, b.y);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, off));
        dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
    }
    return !band_culled(fp, dmin, dmax, p, g, st);
}

template <class Vol, bool FIRST, int ZB = kZB>
__device__ __forceinline__ void integrate_at(const Vol& vol, const float2* __restrict__ tab,
                                             const State* __restrict__ st, const Grid& g, const IntegrateParams& p,
                                             int bx, int by, int bz)
{
    const int x = bx * kIntTx + threadIdx.x;
    const int y = by * kIntTy + threadIdx.y;
    if (x >= g.dx || y >= g.dy) return;
    const int z0 = bz * p.zchunk;
    const int z1 = min(z0 + p.zchunk, g.dz);
    const int H = p.H, W = p.W;
    const float fx = p.fx, fy = p.fy, cx = p.cx, cy = p.cy;
    float ti[12], tx, ty, tz, ax, ay, az;
    load_pose(st, ti, tx, ty, tz, ax, ay, az);
    const float vcx = centre(x, g.sx, g.vd), vcy = centre(y, g.sy, g.vd);
    // the first two products of each row of T^-1 c and of the in-front dot product and
    // |c - t|^2 are the same along the column (left-to-right evaluation)
    const float a0 = ti[0] * vcx + ti[1] * vcy;
    const float a1 = ti[4] * vcx + ti[5] * vcy;
    const float a2 = ti[8] * vcx + ti[9] * vcy;
    const float tdx = vcx - tx, tdy = vcy - ty;
    const float f0 = ax * tdx + ay * tdy;
    const float m0 = tdx * tdx + tdy * tdy;
    const long long rbase = ((long long)x * g.dy + y) * g.dz;
    // the reference's guard compares the thread index with the voxel count in float, so
    // the last z-fastest indices are never integrated; only the last columns get there
    const bool may_skip = rbase + z1 > p.skip_from;
    const int zstride = g.dx * g.dy;  // < 2^31 voxels (checked at kf_create)
    int lin = (z0 * g.dy + y) * g.dx + x;
    // a voxel projects to a pixel of the image iff q = px/pz lies in [0.5, W + 0.5) (and
    // likewise for v); q_approx = px * rcp.approx(pz) is within 2^-21 |q| of the IEEE
    // quotient, so a voxel whose q_approx is outside the range widened by that bound is
    // outside exactly and needs neither division (NaN compares false and falls through)
    const float ulo = 0.5f - 1e-3f, uhi = (float)W + 0.5f + 1e-3f * (float)W;
    const float vlo = 0.5f - 1e-3f, vhi = (float)H + 0.5f + 1e-3f * (float)H;
    const float inv_trunc = 1.f / g.trunc;
    // The column segment in batches of ZB voxels: a batch first runs every voxel's tests
    // up to its pixel, then issues the table loads of the voxels that reach one together,
    // then the volume loads of the voxels that are updated, so that a thread's loads
    // overlap instead of following one another.  Each voxel is read and written by its
    // own thread only, so the order changes no value.  (The listed boxes' pass is a
    // per-box latency chain: 41.9 against 45.6 us per c1 frame for batches of 4 in 16-voxel
    // segments, 36.1 against 37.3 us for one batch of 8 in 8-voxel segments.)
    for (int zb = z0; zb < z1; zb += ZB, lin += ZB * zstride) {
        int pix[ZB];
#pragma unroll
        for (int k = 0; k < ZB; ++k) {
            const int z = zb + k;
            pix[k] = -1;
            if (z >= z1 || (may_skip && rbase + z >= p.skip_from)) continue;
            const float vcz = centre(z, g.sz, g.vd);
            const float tdz = vcz - tz;
            const float front = f0 + az * tdz;
            if (!(front > 0)) continue;
            const float lx = (a0 + ti[2] * vcz) + ti[3];
            const float ly = (a1 + ti[6] * vcz) + ti[7];
            const float lz = (a2 + ti[10] * vcz) + ti[11];
            const float px = fx * lx + cx * lz;
            const float py = fy * ly + cy * lz;
            float r;
            asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(lz));
            const float qu = px * r, qv = py * r;
            if (qu < ulo || qu > uhi || qv < vlo || qv > vhi) continue;
            const int u = (int)roundf(px / lz);
            const int v = (int)roundf(py / lz);
            if (u < 1 || u > W || v < 1 || v > H) continue;
            pix[k] = (v - 1) * W + (u - 1);
        }
        float2 e[ZB];
#pragma unroll
        for (int k = 0; k < ZB; ++k) e[k] = pix[k] >= 0 ? __ldg(tab + pix[k]) : make_float2(qnan(), 0.f);
        float fv[ZB];
        bool upd[ZB];
#pragma unroll
        for (int k = 0; k < ZB; ++k) {
            upd[k] = false;
            fv[k] = 0.f;
            if (isnan(e[k].x)) continue;
            const float tdz = centre(zb + k, g.sz, g.vd) - tz;
            float tm;
            if (Vol::kLean)
                asm("sqrt.approx.f32 %0, %1;" : "=f"(tm) : "f"(m0 + tdz * tdz));
            else
                tm = sqrtf(m0 + tdz * tdz);
            const float frk = e[k].x - e[k].y * tm;
            const bool ahead = frk > 0 && frk <= g.sdf_max;
            const bool behind = frk <= 0 && frk >= g.sdf_min;
            if (!ahead && !behind) continue;
            const float fq = Vol::kLean ? frk * inv_trunc : frk / g.trunc;
            fv[k] = ahead ? fminf(1.f, fq) : fmaxf(-1.f, fq);
            upd[k] = true;
        }
        if (FIRST) {
#pragma unroll
            for (int k = 0; k < ZB; ++k)
                if (upd[k]) vol.store(lin + k * zstride, fv[k], 1.0f);
        } else {
            float t[ZB], w[ZB];
#pragma unroll
            for (int k = 0; k < ZB; ++k) {
                t[k] = w[k] = 0.f;
                if (upd[k]) vol.load(lin + k * zstride, t[k], w[k]);
            }
#pragma unroll
            for (int k = 0; k < ZB; ++k) {
                if (!upd[k]) continue;
                const float tk = isnan(t[k]) ? 0.0f : t[k];
                const float wk = isnan(w[k]) ? 0.0f : w[k];
                if (Vol::kLean) {
                    float rw;
                    asm("rcp.approx.f32 %0, %1;" : "=f"(rw) : "f"(wk + 1.0f));
                    vol.store(lin + k * zstride, fmaf(wk, tk, fv[k]) * rw, wk + 1.0f);
                } else {
                    vol.store(lin + k * zstride, (wk * tk + 1.0f * fv[k]) / (wk + 1.0f), wk + 1.0f);
                }
            }
        }
    }
}

// One block per box (the batched scenes).  Warp 0 decides whether the box can hold an
// updated voxel; a dead box's other warps do nothing but wait for that decision.
template <class Vol, bool FIRST>
__device__ __forceinline__ void integrate_box(const Vol& vol, const float2* __restrict__ tab,
                                              const State* __restrict__ st, const Grid& g, const IntegrateParams& p,
                                              int bx, int by, int bz)
{
    __shared__ int s_live;
    if (threadIdx.y == 0) {
        const bool live = box_live(bx, by, bz, threadIdx.x, g, st, tab + p.H * p.W, p);
        if (threadIdx.x == 0) s_live = live;
    }
    __syncthreads();
    if (s_live) integrate_at<Vol, FIRST>(vol, tab, st, g, p, bx, by, bz);
}

// ---- box marks from the depth tiles (single-scene integration) ----
//
// Which boxes can hold an updated voxel is decided from the pixels' side: a voxel is
// updated only through a pixel (u, v) with a depth D, and then (a) its projection rounds
// to (u, v), so its centre lies in that pixel's frustum widened by half a pixel and by
// the projection's rounding error, and (b) its camera depth lz lies in the band of D
// (band_culled's two tests, each false for it).  For each 8x8 depth tile with (dmin,
// dmax) of its nonzero depths, every such voxel lies in the tile's frustum between the
// camera depths z_a and z_b of those tests; the frustum is cut into slabs of kSlab mm,
// each slab (a convex hexahedron) lies in the box spanned by its eight corners in the
// world, and every integration box that overlaps that (widened) box is marked (plain
// stores of 1).  A compaction pass then lists the marked boxes and clears their marks,
// so every integration starts from unmarked boxes.  Near the camera (lz below kNearZ)
// the pixel margin grows without bound, so when some tile's band reaches below kNearZ
// the boxes within kNearR of the camera centre are listed too (the compaction tests
// each box against the camera).
constexpr float kSlab = 80.f;     // mm of camera depth per slab
constexpr int kMaxSlabs = 512;    // per tile and side (thicker slabs beyond)
constexpr int kMarkLanes = 8;     // lanes per depth tile (slabs over them)

constexpr float kNearZ = 100.f;   // slabs start at this camera depth
constexpr float kNearR = 250.f;   // mm around the camera centre listed when a band reaches kNearZ
                                  // (at least kNearZ times the largest ray norm)

__device__ __forceinline__ void mark_world_box(float3 lo, float3 hi, const Grid& g, unsigned* __restrict__ mark,
                                               int zchunk, int nbx, int nby)
{
    // the grid's extent with a voxel to spare (the conversions below stay in range); NaN
    // corners (a NaN pose, which updates nothing) leave lo > hi
    const float gx0 = ((float)g.sx - 1.f) * g.vd, gx1 = ((float)(g.sx + g.dx) + 1.f) * g.vd;
    const float gy0 = ((float)g.sy - 1.f) * g.vd, gy1 = ((float)(g.sy + g.dy) + 1.f) * g.vd;
    const float gz0 = ((float)g.sz - 1.f) * g.vd, gz1 = ((float)(g.sz + g.dz) + 1.f) * g.vd;
    if (!(lo.x <= gx1 && hi.x >= gx0 && lo.y <= gy1 && hi.y >= gy0 && lo.z <= gz1 && hi.z >= gz0)) return;
    lo = make_float3(fmaxf(lo.x, gx0), fmaxf(lo.y, gy0), fmaxf(lo.z, gz0));
    hi = make_float3(fminf(hi.x, gx1), fminf(hi.y, gy1), fminf(hi.z, gz1));
    // voxel i's centre along x is (i + sx) vd + vd / 2: the voxels with centres in
    // [lo, hi] (the floor and ceiling are already outward; lo and hi carry the corners'
    // rounding margin, and the quotients' own error is below 1e-3 voxel)
    const float ivd = 1.f / g.vd;
    const int i0 = max(0, (int)floorf((lo.x - 0.5f * g.vd) * ivd) - g.sx);
    const int i1 = min(g.dx - 1, (int)ceilf((hi.x - 0.5f * g.vd) * ivd) - g.sx);
    const int j0 = max(0, (int)floorf((lo.y - 0.5f * g.vd) * ivd) - g.sy);
    const int j1 = min(g.dy - 1, (int)ceilf((hi.y - 0.5f * g.vd) * ivd) - g.sy);
    const int k0 = max(0, (int)floorf((lo.z - 0.5f * g.vd) * ivd) - g.sz);
    const int k1 = min(g.dz - 1, (int)ceilf((hi.z - 0.5f * g.vd) * ivd) - g.sz);
    if (i0 > i1 || j0 > j1 || k0 > k1) return;
    // the boxes holding the range
    const int x0 = i0 / kIntTx, y0 = j0 / kIntTy, z0 = k0 / zchunk;
    const int nx = i1 / kIntTx - x0 + 1, ny = j1 / kIntTy - y0 + 1, nz = k1 / zchunk - z0 + 1;
    for (int f = 0; f < nx * ny * nz; ++f)
        mark[((z0 + f / (nx * ny)) * nby + y0 + (f / nx) % ny) * nbx + x0 + f % nx] = 1u;
}

// kMarkLanes threads per depth tile, the tile's slabs over them; a tile whose band
// reaches below kNearZ sets mark_near, and the compaction then lists the boxes around
// the camera too
__global__ void __launch_bounds__(256) integrate_mark_kernel(const float2* __restrict__ tab, State* st, Grid g,
                                                             IntegrateParams p, unsigned* __restrict__ mark, int nbx,
                                                             int nby)
{
    wait_for_producer();
    // the compaction may be scheduled now; it waits for this kernel before reading marks
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int lane = threadIdx.x % kMarkLanes;
    const int tile = blockIdx.x * (256 / kMarkLanes) + threadIdx.x / kMarkLanes;
    const int ntx = bound_tiles_x(p.W), tiles = ntx * ((p.H + kBoundTile - 1) / kBoundTile);
    float T[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) T[k] = st->T[k];
    const float tmax = fmaxf(fmaxf(fabsf(T[3]), fabsf(T[7])), fabsf(T[11]));
    // the margins below hold for a rotation within kRigidTol of orthonormal; a pose
    // further off has every box listed
    if (blockIdx.x == 0 && threadIdx.x == 0 && rigid_error(T) > kRigidTol) st->mark_all = 1u;
    if (tile >= tiles) return;
    const float2 b = tab[p.H * p.W + tile];
    const float dmin = b.x, dmax = b.y;
    if (!(dmin <= dmax)) return;  // no pixel with depth in this tile
    // band_culled's margins: a voxel updated through a pixel with depth D in [dmin, dmax]
    // has z_a <= lz <= z_b (its two tests rearranged for lz); widened by 0.1 % and 1 mm for
    // the float evaluation of these bounds (a few units in the last place) and a rotation
    // up to kRigidTol off orthonormal (a factor within 1 +- 2 kRigidTol)
    const float eps_t = 0x1p-18f * (tmax + 4.f * p.lam_max + 1.f);
    const float abs_t = 0x1p-19f * tmax + 1.f;
    const float hi_band = fmaxf(g.sdf_max, 0.f), lo_band = fminf(g.sdf_min, 0.f);
    const float z_a = (dmin * (1.f - eps_t) - hi_band - 2.f * abs_t) / ((1.f + p.depth_eps) * (1.f + eps_t)) * 0.999f - 1.f;
    // (for a camera some hundreds of metres from the origin eps_t nears 1 and z_b has no
    // bound of its own; the grid's far side below bounds the slabs then)
    const float den_b = (1.f - p.depth_eps) * (1.f - eps_t);
    const float z_b = den_b > 0.5f ? (dmax * (1.f + eps_t) - lo_band + 2.f * abs_t) / den_b * 1.001f + 1.f : INFINITY;
    if (z_a < kNearZ && lane == 0) st->mark_near = 1u;  // the boxes around the camera too
    // A voxel's |lz| is at most its distance from the camera centre (with 1 % for a pose
    // a little off orthonormal and for the rounding of lz), and no voxel centre lies
    // farther than the grid's farthest corner centre: the slabs end there, so a depth of
    // 1e30 or inf costs no more slabs than the grid's own depth.  A NaN pose updates
    // nothing.
    float far2 = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int s0 = a == 0 ? g.sx : a == 1 ? g.sy : g.sz, n = a == 0 ? g.dx : a == 1 ? g.dy : g.dz;
        const float t = T[4 * a + 3];
        const float d = fmaxf(fabsf(((float)s0 + 0.5f) * g.vd - t), fabsf(((float)(s0 + n) - 0.5f) * g.vd - t));
        far2 += d * d;
    }
    const float z_far = sqrtf(far2) * 1.01f + 2.f * g.vd + 1.f;
    if (isnan(z_far)) return;
    const float z_lo = fmaxf(z_a, kNearZ), z_hi = fminf(z_b, z_far);
    if (!(z_hi > z_lo)) return;
    const float span = z_hi - z_lo;
    if (!(span < 1e30f)) {  // no finite bound (an infinite translation): every box
        if (lane == 0) st->mark_all = 1u;
        return;
    }
    // slabs of kSlab, thicker where the span would need more than kMaxSlabs of them
    const float slab = fmaxf(kSlab, span * (1.f / (float)kMaxSlabs));
    const int nslab = min(kMaxSlabs, (int)ceilf(span / slab));
    // rounding error of a voxel's camera coordinates (integrate_at's evaluation): at
    // most 2^-19 of a generous bound on their terms' magnitudes, the grid's extent plus
    // the camera's distance from the origin; the pixel margin is taken at the nearest
    // slab depth z_lo, where it is largest: one pixel for the rounding to a pixel centre
    // plus the projection's error
    const float ext = (float)(max(max(abs(g.sx), abs(g.sx + g.dx)), max(max(abs(g.sy), abs(g.sy + g.dy)),
                                                                      max(abs(g.sz), abs(g.sz + g.dz))))) *
                      g.vd;
    const float err_l = 0x1p-19f * 4.f * (ext + tmax);
    const float mpx = 1.f + (fmaxf(p.fx, p.fy) + fmaxf(fabsf(p.cx), fabsf(p.cy)) + (float)max(p.W, p.H) + 10.f) *
                                err_l / z_lo + 1e-3f;
    // the tile's pixels (1-based) span [x0 + 0.5, x0 + 8.5] in projected coordinates; the
    // four corner rays (camera x / z, y / z) of that range widened by mpx, in the world
    const float u_a = (float)((tile % ntx) * kBoundTile) + 0.5f, v_a = (float)((tile / ntx) * kBoundTile) + 0.5f;
    const float rx0 = (u_a - mpx - p.cx) / p.fx, rx1 = (u_a + 8.f + mpx - p.cx) / p.fx;
    const float ry0 = (v_a - mpx - p.cy) / p.fy, ry1 = (v_a + 8.f + mpx - p.cy) / p.fy;
    float3 wr[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float X = (c & 1) ? rx1 : rx0, Y = (c & 2) ? ry1 : ry0;
        wr[c] = make_float3(T[0] * X + T[1] * Y + T[2], T[4] * X + T[5] * Y + T[6], T[8] * X + T[9] * Y + T[10]);
    }
    const float rmax = fmaxf(fmaxf(fabsf(rx0), fabsf(rx1)), fmaxf(fabsf(ry0), fabsf(ry1)));
    // Voxels behind the camera.  The in-front test is a . (c - t) > 0 with a = R ca,
    // ca = K^-1 (cy, cx, 1) (the reference's swapped principal point), i.e. ca . l > 0 for
    // the voxel's camera coordinates l = lz (X, Y, 1): lz s(X, Y) > 0 with s = ca_x X +
    // ca_y Y + 1.  A voxel behind the camera (lz < 0) projects, mirrored, to the pixel of
    // (X, Y) as well, and passes where s < 0: with a wide field of view and cx far from
    // cy the reference updates such voxels (|lz| in the same band).  The test's rounding
    // (the axis against the translation, the dot product) is below 2^-19 (|ca| + 2 tmax)
    // |lz| lam_max, and a rotation off orthonormal by up to kRigidTol moves the test by
    // 2 kRigidTol |ca| |lz| lam_max at most; where s exceeds twice their sum over the
    // tile's widened rays (s is linear: its minimum is at a corner) no voxel behind the
    // camera is updated through the tile; elsewhere the slabs are marked mirrored too (z
    // from -z_hi to -z_lo).
    const float ca_x = (p.cy - p.cx) / p.fx, ca_y = (p.cx - p.cy) / p.fy;
    const float s_min = 1.f + fminf(ca_x * rx0, ca_x * rx1) + fminf(ca_y * ry0, ca_y * ry1);
    const float ca_n = 1.f + fabsf(ca_x) + fabsf(ca_y);
    const float s_margin = (0x1p-18f * (ca_n + 2.f * tmax) + 4.f * kRigidTol * ca_n) * p.lam_max + 1e-3f;
    const int nside = s_min > s_margin ? 1 : 2;
    for (int k = lane; k < nside * nslab; k += kMarkLanes) {
        const int ks = k < nslab ? k : k - nslab;
        const float sgn = k < nslab ? 1.f : -1.f;
        const float za = z_lo + (float)ks * slab;
        const float zb = ks == nslab - 1 ? z_hi : fminf(z_lo + (float)(ks + 1) * slab, z_hi);
        // the slab's corners t + z R (x/z, y/z, 1) for z = za, zb (or -za, -zb); each
        // coordinate is within a relative 2^-20 of its terms' magnitudes, covered by e
        // (and a millimetre)
        float3 lo = make_float3(INFINITY, INFINITY, INFINITY), hi = make_float3(-INFINITY, -INFINITY, -INFINITY);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float z = sgn * ((c & 4) ? zb : za);
            const float3 w = wr[c & 3];
            const float wx = w.x * z + T[3], wy = w.y * z + T[7], wz = w.z * z + T[11];
            lo = make_float3(fminf(lo.x, wx), fminf(lo.y, wy), fminf(lo.z, wz));
            hi = make_float3(fmaxf(hi.x, wx), fmaxf(hi.y, wy), fmaxf(hi.z, wz));
        }
        const float e = 0x1p-17f * ((2.f * rmax + 1.f) * 2.f * zb + tmax) + 1.f;
        lo = make_float3(lo.x - e, lo.y - e, lo.z - e);
        hi = make_float3(hi.x + e, hi.y + e, hi.z + e);
        mark_world_box(lo, hi, g, mark, p.zchunk, nbx, nby);
    }
}

// The marked boxes in order, as a list after the marks (mark + nboxes), and the marks
// cleared: one thread per box, one atomic per warp for the warp's marked boxes.
__global__ void __launch_bounds__(256) integrate_list_kernel(State* st, unsigned* __restrict__ mark, Grid g,
                                                             int zchunk, int nbx, int nby, int nboxes, float near_r)
{
    wait_for_producer();
    // integration may be scheduled now; it waits for this kernel before reading the list
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool m = b < nboxes && (mark[b] != 0u || st->mark_all != 0u);
    if (!m && b < nboxes && st->mark_near) {
        // the box's voxel centres against the camera centre widened by near_r (and two
        // voxels for the rounding of both)
        const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
        const float r = near_r + 2.f * g.vd;
        const auto overlaps = [&](int i0, int n, int s0, float c) {
            const float lo = ((float)(i0 + s0) + 0.5f) * g.vd, hi = ((float)(i0 + n - 1 + s0) + 0.5f) * g.vd;
            return hi >= c - r && lo <= c + r;
        };
        m = overlaps(bx * kIntTx, kIntTx, g.sx, st->T[3]) && overlaps(by * kIntTy, kIntTy, g.sy, st->T[7]) &&
            overlaps(bz * zchunk, zchunk, g.sz, st->T[11]);
    }
    const unsigned ball = __ballot_sync(0xffffffffu, m);
    if (!ball) return;
    unsigned base = 0u;
    if (lane == 0) base = atomicAdd(&st->mark_count, (unsigned)__popc(ball));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (m) {
        mark[nboxes + base + __popc(ball & ((1u << lane) - 1u))] = (unsigned)b;
        mark[b] = 0u;
    }
}

// Persistent: the blocks take the boxes on the mark list in strides of the grid (the
// list is in box order); a block of 32 x 8 threads updates one 32 x 8 x 8 box at a time,
// a thread its 8-voxel column segment with the loads of all eight issued together (no
// spills at four blocks per SM).
constexpr int kListZB = 8;

template <class Vol, bool FIRST>
__global__ void __launch_bounds__(kIntTx* kIntTy, 4) integrate_kernel(Vol vol, const float2* __restrict__ tab,
                                                                   const State* __restrict__ st, Grid g,
                                                                   IntegrateParams p,
                                                                   const unsigned* __restrict__ mark, int nbx, int nby,
                                                                   int nboxes)
{
    wait_for_producer();
    // the ray cast may be scheduled once every block has started; it waits for this
    // kernel before reading the volume
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const unsigned n = st->mark_count;
    const unsigned* list = mark + nboxes;
    for (unsigned i = blockIdx.x; i < n; i += gridDim.x) {
        const int box = (int)list[i];
        integrate_at<Vol, FIRST, kListZB>(vol, tab, st, g, p, box % nbx, (box / nbx) % nby, box / (nbx * nby));
    }
}

__device__ __forceinline__ VolF32 scene_volume(const SceneDev& d, VolF32*) { return VolF32{d.tsdf, d.weight}; }
__device__ __forceinline__ VolF16 scene_volume(const SceneDev& d, VolF16*) { return VolF16{d.vol16}; }

// every scene's integration: blockIdx.y picks the scene, blockIdx.x its box; scenes with
// fewer boxes than the largest return early
template <class Vol, bool FIRST>
__global__ void __launch_bounds__(kIntTx* kIntTy, 5) integrate_batch_kernel(const SceneDev* __restrict__ scenes, int zchunk)
{
    wait_for_producer();
    const SceneDev& d = scenes[blockIdx.y];
    const Grid& g = d.grid;
    const int nbx = (g.dx + kIntTx - 1) / kIntTx, nby = (g.dy + kIntTy - 1) / kIntTy, nbz = (g.dz + zchunk - 1) / zchunk;
    const int t = blockIdx.x;
    if (t >= nbx * nby * nbz) return;
    const Vol vol = scene_volume(d, (Vol*)nullptr);
    integrate_box<Vol, FIRST>(vol, d.tab, d.st, g, scene_params(d, zchunk), t % nbx, (t / nbx) % nby,
                              t / (nbx * nby));
}

// every scene's integration as a persistent launch: blocks take boxes one at a time from
// one counter over all scenes' boxes (scene s owns boxes [int_start of s, int_start of
// s + 1)), so the scenes' live boxes share the SMs without blocks for the boxes smaller
// grids do not have; counter: two unsigneds, zero between launches (the last block to
// leave resets them)
template <class Vol, bool FIRST>
__global__ void __launch_bounds__(kIntTx* kIntTy, 5) integrate_batch_persist_kernel(
    const SceneDev* __restrict__ scenes, int n_scenes, int zchunk, unsigned total, unsigned* counter)
{
    wait_for_producer();
    __shared__ unsigned s_box;
    const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
    for (;;) {
        __syncthreads();  // the previous box is done with s_box and the cull flag
        if (lead) s_box = atomicAdd(counter, 1u);
        __syncthreads();
        const unsigned box = s_box;
        if (box >= total) {
            if (lead && atomicAdd(counter + 1, 1u) == gridDim.x - 1) {
                counter[0] = 0u;
                counter[1] = 0u;
            }
            return;
        }
        int s = 0;
        while (s + 1 < n_scenes && box >= (unsigned)scenes[s + 1].int_start) ++s;
        const SceneDev& d = scenes[s];
        const Grid& g = d.grid;
        const int nbx = (g.dx + kIntTx - 1) / kIntTx, nby = (g.dy + kIntTy - 1) / kIntTy;
        const int t = (int)(box - (unsigned)d.int_start);
        const Vol vol = scene_volume(d, (Vol*)nullptr);
        integrate_box<Vol, FIRST>(vol, d.tab, d.st, g, scene_params(d, zchunk), t % nbx, (t / nbx) % nby,
                                  t / (nbx * nby));
    }
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
// Called by all 32 lanes of a warp together (the walk's votes take the full mask); a
// lane without a ray passes D = 0.
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
    // every lane of the warp walks (the group votes below take the full mask); a lane
    // without a ray (no depth, or a ray that misses the grid) starts finished
    const bool walks = D != 0 && inside;
    if (tmin < 0) tmin = 0;
    const float3 s = make_float3(org.x + tmin * dir.x, org.y + tmin * dir.y, org.z + tmin * dir.z);
    const float3 box = make_float3(hi.x - lo.x, hi.y - lo.y, hi.z - lo.z);
    int ix = (int)floorf(((s.x - lo.x) / box.x) * L) + 1;
    int iy = (int)floorf(((s.y - lo.y) / box.y) * Wd) + 1;
    int iz = (int)floorf(((s.z - lo.z) / box.z) * Hz) + 1;
    if (!walks) ix = iy = iz = 1;
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
    // The walk visits positions 0, 1, 2, ... until the first one outside the loop bounds
    // (:203-205).  The start is tested once; after it every index moves in one fixed
    // direction, so each axis can leave the bounds only on one side, and a position is
    // inside iff the steps each axis has left before that side, r = (n - 2) - i going up
    // or i - 1 going down, are all >= 0 -- one OR and one sign test per position, and
    // once outside a walk stays outside.
    const bool start_in = walks && inside_grid(ix, iy, iz);
    int rx = sx > 0 ? (L - 2) - ix : ix - 1;
    int ry = sy > 0 ? (Wd - 2) - iy : iy - 1;
    int rz = sz > 0 ? (Hz - 2) - iz : iz - 1;
    if (!start_in) rx = -1;
    // The stepping never depends on the loaded values, only the termination does, so a
    // lead walker with the same arithmetic runs kAhead steps in front: at each position
    // it issues the voxel's load into a register ring and records, beside it, the
    // position's linear index and a code, the linear-index delta of the step from it
    // (the Amanatides-Woo step, :384-417: the same three comparisons pick the axis;
    // dlx, dly, dlz are distinct and nonzero since every side is at least 3 voxels) when
    // the position is inside the bounds, else 0.  The trailing walk consumes value,
    // index and code in order and keeps no indices of its own.  The reference's XY..ZY
    // (the other two indices at the last step along x, y, z) are kept as the linear
    // index of the position each last such step left from (-1 before the first: the
    // reference's never-assigned zeros) and decoded after the walk.  The lead loads only
    // voxels inside the bounds.
    constexpr int kAhead = 4;
    int ali = li;
    float3 atm = tm;
    // The axis choice as predicates and selects, with no branch: lanes of a warp step
    // along different axes, and a three-way branch per step diverged (61.6 -> 58.0 us
    // per c1 frame without it).
    auto lead_step = [&]() -> int {
        const bool xy = atm.x < atm.y, xz = atm.x < atm.z, yz = atm.y < atm.z;
        const bool px = xy && xz, py = !xy && yz, pz = !px && !py;
        rx -= (int)px;
        ry -= (int)py;
        rz -= (int)pz;
        const float nx = atm.x + td.x, ny = atm.y + td.y, nz = atm.z + td.z;
        atm.x = px ? nx : atm.x;
        atm.y = py ? ny : atm.y;
        atm.z = pz ? nz : atm.z;
        const int d = px ? dlx : (py ? dly : dlz);
        ali += d;
        return d;
    };
    typename View::Raw ring[kAhead];
    int ring_li[kAhead];
    int code[kAhead];
#pragma unroll
    for (int k = 0; k < kAhead; ++k) {
        const bool in = (rx | ry | rz) >= 0;
        ring[k] = in ? vol.raw(ali) : typename View::Raw(0);
        ring_li[k] = ali;
        const int step = lead_step();
        code[k] = in ? step : 0;
    }
    float prev = 0.0f;
    float crossing = 0.f;  // the negative value met right after a positive one, or 0
    int rec_x = -1, rec_y = -1, rec_z = -1;
    bool done = !start_in;
    // Steps run in groups of kAhead without branches; the warp leaves the loop when
    // every lane's walk has ended, and a lane whose walk has ended steps on with its
    // results frozen and its lead outside the bounds (no loads).  Every step moves one
    // index one step in a fixed direction, so a walk ends within L + Wd + Hz steps; the
    // bound only makes that explicit.
    for (int guard = 0; guard < L + Wd + Hz + 4; guard += kAhead) {
        // A group in which every walking lane has kAhead positions inside the bounds, none
        // of negative value, after a previous value that is not negative, advances through
        // all of them by the reference's tests: each of :207-222 needs a negative value
        // before or at the position, and so does a zero crossing.  When the whole warp is
        // in that case, only the lead and the axis records run.
        unsigned key = View::negative_key(ring[0]);
        bool all_in = code[0] != 0;
#pragma unroll
        for (int k = 1; k < kAhead; ++k) {
            key = min(key, View::negative_key(ring[k]));
            all_in = all_in && code[k] != 0;
        }
        const bool easy = done || (!(prev < 0.f) && all_in && key >= View::kNegativeKeys);
        if (__all_sync(0xffffffffu, easy)) {
            const typename View::Raw last = ring[kAhead - 1];
#pragma unroll
            for (int k = 0; k < kAhead; ++k) {
                const int c = code[k];  // 0 for a finished lane: no records change
                const int here = ring_li[k];
                const bool in = (rx | ry | rz) >= 0;
                if (in) ring[k] = vol.raw(ali);  // outside the bounds: a stale value, unused (code 0)
                ring_li[k] = ali;
                const int step = lead_step();
                code[k] = in ? step : 0;
                rec_x = c == dlx ? here : rec_x;
                rec_y = c == dly ? here : rec_y;
                rec_z = c == dlz ? here : rec_z;
            }
            prev = View::decode(last);  // unused once the walk has ended
        } else {
#pragma unroll
            for (int k = 0; k < kAhead; ++k) {
                const int c = code[k];
                const float cur = View::decode(ring[k]);
                const int here = ring_li[k];
                const bool in = (rx | ry | rz) >= 0;
                if (in) ring[k] = vol.raw(ali);
                ring_li[k] = ali;
                const int step = lead_step();
                code[k] = in ? step : 0;
                // the position ends the walk if it is outside the bounds, or by the
                // reference's four tests (:207-222, mutually exclusive in prev), or as
                // the zero crossing (a negative value right after a positive one)
                const bool live = !done && c != 0;
                const bool stop = prev < 0.f ? !(cur <= 0.f) : (isnan(prev) && cur < 0.f);
                const bool cross = live && !stop && prev > 0.f && cur < 0.f;
                crossing = cross ? cur : crossing;
                li = cross ? here : li;
                const bool adv = live && !stop && !cross;
                done = !adv;
                prev = adv ? cur : prev;
                rec_x = (adv && c == dlx) ? here : rec_x;
                rec_y = (adv && c == dly) ? here : rec_y;
                rec_z = (adv && c == dlz) ? here : rec_z;
            }
            if (done) {
                // the lead's positions queued behind the end carry no records, and it
                // issues no further loads
#pragma unroll
                for (int k = 0; k < kAhead; ++k) code[k] = 0;
                rx = -1;
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
    }
    if (!(crossing < 0.f)) return;
    // the crossing's position and the recorded indices, 1-based as in the reference
    // (linear indices are non-negative and below 2^31; the divisions are multiply-highs)
    {
        const int q = div_by(li, g.qdx), r = div_by(q, g.qdy);
        ix = li - q * L + 1;
        iy = q - r * Wd + 1;
        iz = r + 1;
    }
    int XY = 0, XZ = 0, YX = 0, YZ = 0, ZX = 0, ZY = 0;
    if (rec_x >= 0) {
        const int q = div_by(rec_x, g.qdx), r = div_by(q, g.qdy);
        XY = q - r * Wd + 1;
        XZ = r + 1;
    }
    if (rec_y >= 0) {
        const int q = div_by(rec_y, g.qdx);
        YX = rec_y - q * L + 1;
        YZ = div_by(q, g.qdy) + 1;
    }
    if (rec_z >= 0) {
        const int q = div_by(rec_z, g.qdx);
        ZX = rec_z - q * L + 1;
        ZY = q - div_by(q, g.qdy) * Wd + 1;
    }
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
        // every lane traces (a lane off the image or without depth walks no steps)
        const bool pixel = px < cam.W && py < cam.H;
        const int i = py * cam.W + px;
        float4 op = make_float4(0.f, 0.f, 0.f, 0.f), on = op;
        int oh = -1;
        const float D = pixel ? depth[i] : 0.f;
        trace(vol, (float)px + 1.0f, (float)py + 1.0f, D, cam.Ki, T, g, c_flip, op, on, oh);
        if (!pixel) continue;
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
        const bool pixel = px < cam.W && py < cam.H;
        float T[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) T[k] = d.st->T[k];
        const int i = py * cam.W + px;
        float4 op = make_float4(0.f, 0.f, 0.f, 0.f), on = op;
        int oh = -1;
        const float D = pixel ? d.depth[0][i] : 0.f;
        trace(scene_view(d, (View*)nullptr), (float)px + 1.0f, (float)py + 1.0f, D, cam.Ki, T, d.grid, d.st->c_flip,
              op, on, oh);
        if (!pixel) continue;
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

// once per device, outside any stream capture: sizes the persistent integration grid
int integrate_blocks()
{
    static int blocks[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152 * 4;
    if (!blocks[dev]) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, integrate_kernel<VolF16, false>, kIntTx * kIntTy, 0);
        blocks[dev] = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 4);
    }
    return blocks[dev];
}

void launch_integrate_prep(const float* depth, float2* tab, const Camera& cam, State* st, cudaStream_t s)
{
    launch_pdl(integrate_prep_kernel, dim3((depth_bound_tiles(cam.H, cam.W) + 7) / 8), dim3(256), 0, s, depth, tab,
               cam, st);
}

int depth_bound_tiles(int H, int W)
{
    return ((W + kBoundTile - 1) / kBoundTile) * ((H + kBoundTile - 1) / kBoundTile);
}

float depth_band_eps(const Camera& cam)
{
    // |tm / |R lambda| - lz| / lz <= 2 |a| dx + dx^2 + 2 |b| dy + dy^2 with dx = 1/(2 fx),
    // dy = 1/(2 fy) and |a|, |b| the largest |x/z|, |y/z| of a voxel projecting into the
    // image; doubled, plus 1e-4 for float rounding
    const float fx = cam.K[0], fy = cam.K[4], cx = cam.K[2], cy = cam.K[5];
    const float a = (fmaxf(cx, (float)cam.W + 1.f - cx) + 1.f) / fx, b = (fmaxf(cy, (float)cam.H + 1.f - cy) + 1.f) / fy;
    const float dx = 0.5f / fx, dy = 0.5f / fy;
    return 2.f * (2.f * a * dx + dx * dx + 2.f * b * dy + dy * dy) + 1e-4f;
}

float ray_norm_max(const Camera& cam)
{
    // |K^-1 (u, v, 1)| is convex in (u, v): its largest value is at a corner pixel
    double m = 0.0;
    for (int cu = 0; cu < 2; ++cu)
        for (int cv = 0; cv < 2; ++cv) {
            const double u = cu ? cam.W : 1, v = cv ? cam.H : 1;
            double n = 0.0;
            for (int r = 0; r < 3; ++r) {
                const double c = (double)cam.Ki[3 * r] * u + (double)cam.Ki[3 * r + 1] * v + (double)cam.Ki[3 * r + 2];
                n += c * c;
            }
            m = std::max(m, std::sqrt(n));
        }
    return (float)(m * 1.01 + 1e-3);
}

namespace {
constexpr int kZChunk = 8;  // voxels along z per box of the single-scene integration

IntegrateParams host_params(const Camera& cam, int zchunk, long long skip_from)
{
    return IntegrateParams{cam.K[0], cam.K[4], cam.K[2], cam.K[5], cam.H, cam.W, zchunk, skip_from,
                           depth_band_eps(cam), ray_norm_max(cam)};
}

template <class Vol>
void integrate_launch(Vol vol, const float2* tab, const State* st, const Grid& g, const Camera& cam,
                      long long skip_from, bool first, unsigned* mark, cudaStream_t s)
{
    const IntegrateParams p = host_params(cam, kZChunk, skip_from);
    const dim3 block(kIntTx, kIntTy);
    const dim3 grid((g.dx + kIntTx - 1) / kIntTx, (g.dy + kIntTy - 1) / kIntTy, (g.dz + kZChunk - 1) / kZChunk);
    const int nboxes = (int)(grid.x * grid.y * grid.z);
    launch_pdl(integrate_mark_kernel, dim3((depth_bound_tiles(cam.H, cam.W) * kMarkLanes + 255) / 256), dim3(256), 0, s,
               tab, const_cast<State*>(st), g, p, mark, (int)grid.x, (int)grid.y);
    // a voxel updated with camera depth lz < kNearZ lies within kNearZ max|K^-1 (u, v, 1)|
    // of the camera centre (the ray norm at the image's corner pixels, with a 1 % margin
    // that covers the half pixel beyond them)
    const float near_r = std::max(kNearR, kNearZ * p.lam_max);
    launch_pdl(integrate_list_kernel, dim3((nboxes + 255) / 256), dim3(256), 0, s, const_cast<State*>(st), mark, g,
               p.zchunk, (int)grid.x, (int)grid.y, nboxes, near_r);
    const dim3 blocks(integrate_blocks());
    if (first)
        launch_pdl(integrate_kernel<Vol, true>, blocks, block, 0, s, vol, tab, st, g, p, (const unsigned*)mark,
                   (int)grid.x, (int)grid.y, nboxes);
    else
        launch_pdl(integrate_kernel<Vol, false>, blocks, block, 0, s, vol, tab, st, g, p, (const unsigned*)mark,
                   (int)grid.x, (int)grid.y, nboxes);
}
}  // namespace

void launch_integrate_f32(float* tsdf, float* weight, const float2* tab, const State* st, const Grid& g,
                          const Camera& cam, long long skip_from, bool first, unsigned* mark, cudaStream_t s)
{
    integrate_launch(VolF32{tsdf, weight}, tab, st, g, cam, skip_from, first, mark, s);
}

void launch_integrate_f16(__half2* vol, const float2* tab, const State* st, const Grid& g, const Camera& cam,
                          long long skip_from, bool first, unsigned* mark, cudaStream_t s)
{
    integrate_launch(VolF16{vol}, tab, st, g, cam, skip_from, first, mark, s);
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
    launch_pdl(integrate_prep_batch_kernel, dim3((max_pixels / 64 + 7) / 8 + 1, n_scenes), dim3(256), 0, s, scenes);
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

void launch_integrate_batch_persistent(const SceneDev* scenes, int n_scenes, int max_pixels, unsigned total_boxes,
                                       int zchunk, bool f16, bool first, int blocks, unsigned* counter, cudaStream_t s)
{
    launch_pdl(integrate_prep_batch_kernel, dim3((max_pixels / 64 + 7) / 8 + 1, n_scenes), dim3(256), 0, s, scenes);
    const dim3 grid(blocks), block(kIntTx, kIntTy);
    if (f16) {
        if (first)
            launch_pdl(integrate_batch_persist_kernel<VolF16, true>, grid, block, 0, s, scenes, n_scenes, zchunk,
                       total_boxes, counter);
        else
            launch_pdl(integrate_batch_persist_kernel<VolF16, false>, grid, block, 0, s, scenes, n_scenes, zchunk,
                       total_boxes, counter);
    } else {
        if (first)
            launch_pdl(integrate_batch_persist_kernel<VolF32, true>, grid, block, 0, s, scenes, n_scenes, zchunk,
                       total_boxes, counter);
        else
            launch_pdl(integrate_batch_persist_kernel<VolF32, false>, grid, block, 0, s, scenes, n_scenes, zchunk,
                       total_boxes, counter);
    }
}

int integrate_boxes(const Grid& g) { return integrate_tiles(g, kZChunk); }

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
