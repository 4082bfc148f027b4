/*
 * TEST INFRASTRUCTURE -- the CPU oracle (see kf_oracle.h).  Never part of the product.
 *
 * Each function restates one reference kernel body, keeping the reference's
 * expression order so that, built with -ffp-contract=off, every float result rounds
 * exactly as the reference's own code does when compiled the same way.  Citations are
 * to PoChang007/Kinect_Fusion_SLAM (file:line).
 */
#include "kf_oracle.h"
#include "ocv_restated.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* CUDART_PI_F (math_constants.h) as used by voxel_traversal.cu:362 and
 * sensor_pose_estimation.cu:64 */
const float kPiF = 3.141592654f;

struct F3 {
    float x, y, z;
};

/* Get_Normalized, cuda_functions.cuh:1-10 */
inline F3 normalized(F3 v)
{
    float r = 1 / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return F3{v.x * r, v.y * r, v.z * r};
}

/* rows 0..2 of a 4x4 row-major transform applied to a point, reference order
 * ((m0*x + m1*y) + m2*z) + m3 */
inline F3 xform_point(const float* m, F3 p)
{
    return F3{m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}

/* 3x3 row-major times vector */
inline F3 mul3(const float* m, F3 p)
{
    return F3{m[0] * p.x + m[1] * p.y + m[2] * p.z, m[3] * p.x + m[4] * p.y + m[5] * p.z,
              m[6] * p.x + m[7] * p.y + m[8] * p.z};
}

/* voxel centre coordinate, kinfu_pipeline.cpp:53-55: x * voxel_distance + voxel_distance / 2 */
inline float centre(int index, int start, float vd) { return (float)(index + start) * vd + vd / 2.f; }

inline long zfast(long x, long y, long z, long DY, long DZ) { return x * DY * DZ + y * DZ + z; }

}  // namespace

extern "C" {

void kfo_inv3(const float* K, float* Kinv) { ocv_inv3(K, Kinv); }
int kfo_inv4(const float* T, float* Tinv) { return ocv_inv4(T, Tinv); }
void kfo_matmul4(const float* A, const float* B, float* C) { ocv_matmul4(A, B, C); }
int kfo_cholesky6(float* A, float* b) { return ocv_cholesky6(A, b); }

float kfo_icp_angle_deg(float cos_theta) { return std::acos(cos_theta) * (180.0f / kPiF); }

int kfo_raycast_flip(float cos_theta)
{
    double c = cos_theta;
    double angle = std::acos(c) * (180.0f / kPiF);
    return angle > 90 ? 1 : 0;
}

int kfo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* system_utility.cpp:58-68 (uint16 -> float) and :77-85 (cv::inRange inclusive mask) */
void kfo_depth_ingest(const uint16_t* raw, int n, float min_depth, float max_depth, float* out)
{
    for (int i = 0; i < n; ++i) {
        float d = (float)raw[i];
        out[i] = (d >= min_depth && d <= max_depth) ? d : 0.f;
    }
}

/* raw_vertices.cu:3-51 */
void kfo_vertex_normal(int H, int W, const float* depth, const float* Ki, float* vx, float* vy, float* nx,
                       float* ny, float* nz, uint8_t* mask)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H * W; ++i) {
        vx[i] = vy[i] = nx[i] = ny[i] = nz[i] = 0.f;
        mask[i] = 0;
        const int row = i / W, col = i % W;
        if (!(depth[i] != 0 && row != H - 1 && col != W - 1)) continue;
        mask[i] = 1;
        const int down = (row + 1) * W + col;
        const int right = row * W + col + 1;
        if (!(down > 0 && right > 0 && depth[down] != 0 && depth[right] != 0)) continue;
        const float d = depth[i], dd = depth[down], dr = depth[right];
        const float X = (float)(col + 1), Y = (float)(row + 1);
        const float px = d * (Ki[0] * X + Ki[1] * Y + Ki[2]);
        const float py = d * (Ki[3] * X + Ki[4] * Y + Ki[5]);
        const float dx = dd * (Ki[0] * X + Ki[1] * (float)(row + 2) + Ki[2]);
        const float rx = dr * (Ki[0] * (float)(col + 2) + Ki[1] * Y + Ki[2]);
        const float dy = dd * (Ki[3] * X + Ki[4] * (float)(row + 2) + Ki[5]);
        const float ry = dr * (Ki[3] * (float)(col + 2) + Ki[4] * Y + Ki[5]);
        /* (v_down - v) x (v_right - v), raw_vertices.cu:33-38 */
        const float n0 = (dy - py) * (dr - d) - (dd - d) * (ry - py);
        const float n1 = (dd - d) * (rx - px) - (dx - px) * (dr - d);
        const float n2 = (dx - px) * (ry - py) - (dy - py) * (rx - px);
        const float len = std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
        vx[i] = px;
        vy[i] = py;
        nx[i] = n0 / len;
        ny[i] = n1 / len;
        nz[i] = n2 / len;
    }
}

/* projective_tsdf.cu:5-140 */
void kfo_integrate(const kfo_grid* g, int H, int W, const float* depth, const float* K, const float* Ki,
                   const float* T, const float* Ti, float* tsdf, float* weight, int first)
{
    const int DX = g->dims[0], DY = g->dims[1], DZ = g->dims[2];
    const float vd = g->voxel_size, trunc = g->truncated_distance;
    const float smin = g->sdf_minimum, smax = g->sdf_maximum;
    const F3 cam{T[3], T[7], T[11]};
    /* "in front of the camera" direction from K^-1 [K(1,2), K(0,2), 1] (swapped
     * principal point) and twice that, both taken to world, :57-71 */
    const F3 ca = mul3(Ki, F3{K[5], K[2], 1.f});
    const F3 cb{2 * (Ki[0] * K[5] + Ki[1] * K[2] + Ki[2] * 1.f), 2 * (Ki[3] * K[5] + Ki[4] * K[2] + Ki[5] * 1.f),
                2 * (Ki[6] * K[5] + Ki[7] * K[2] + Ki[8] * 1.f)};
    const F3 ga = xform_point(T, ca), gb = xform_point(T, cb);
    const F3 axis{gb.x - ga.x, gb.y - ga.y, gb.z - ga.z};
    /* the kernel's guard `x >= voxel_length * voxel_width * voxel_height` (:14) compares
     * the int thread index with a float product, so indices that round up to the voxel
     * count in float are skipped (the last voxel of the 360x360x300 grid) */
    const float nvox_f = (float)DX * (float)DY * (float)DZ;

#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < DX; ++ix) {
        const float cx = centre(ix, g->start[0], vd);
        for (int iy = 0; iy < DY; ++iy) {
            const float cy = centre(iy, g->start[1], vd);
            for (int iz = 0; iz < DZ; ++iz) {
                const long idx = zfast(ix, iy, iz, DY, DZ);
                if ((float)(int)idx >= nvox_f) continue;
                const F3 c{cx, cy, centre(iz, g->start[2], vd)};
                const F3 local = xform_point(Ti, c);
                const F3 p = mul3(K, local);
                const int u = (int)std::round(p.x / p.z);
                const int v = (int)std::round(p.y / p.z);
                if (!(u > 0 && u <= W && v > 0 && v <= H)) continue;
                const float D = depth[(v - 1) * W + (u - 1)];
                if (!(D != 0)) continue;
                const F3 lam{Ki[0] * u + Ki[1] * v + Ki[2] * 1.f, Ki[3] * u + Ki[4] * v + Ki[5] * 1.f,
                             Ki[6] * u + Ki[7] * v + Ki[8] * 1.f};
                const F3 rs = xform_point(T, lam);
                const F3 rd{T[0] * 2 * lam.x + T[1] * 2 * lam.y + T[2] * 2 * lam.z + T[3],
                            T[4] * 2 * lam.x + T[5] * 2 * lam.y + T[6] * 2 * lam.z + T[7],
                            T[8] * 2 * lam.x + T[9] * 2 * lam.y + T[10] * 2 * lam.z + T[11]};
                const F3 dir{rd.x - rs.x, rd.y - rs.y, rd.z - rs.z};
                const float mag = std::sqrt(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
                const F3 td{c.x - cam.x, c.y - cam.y, c.z - cam.z};
                const float front = axis.x * td.x + axis.y * td.y + axis.z * td.z;
                if (!(front > 0)) continue;
                const float tmag = std::sqrt(td.x * td.x + td.y * td.y + td.z * td.z);
                const F3 pt = xform_point(T, F3{D * lam.x, D * lam.y, D * lam.z});
                const F3 rel{pt.x - cam.x, pt.y - cam.y, pt.z - cam.z};
                const float dist = std::sqrt(rel.x * rel.x + rel.y * rel.y + rel.z * rel.z);
                const float pdepth = dist / mag;
                float frk = pdepth - ((1.f / mag) * tmag);
                const bool ahead = frk > 0 && frk <= smax;
                const bool behind = frk <= 0 && frk >= smin;
                if (!ahead && !behind) continue;
                if (first) {
                    tsdf[idx] = ahead ? std::fmin(1.f, frk / trunc) : std::fmax(-1.f, frk / trunc);
                    weight[idx] = 1.0f;
                } else {
                    if (std::isnan(tsdf[idx])) tsdf[idx] = 0.0f;
                    if (std::isnan(weight[idx])) weight[idx] = 0.0f;
                    frk = ahead ? std::fmin(1.f, frk / trunc) : std::fmax(-1.f, frk / trunc);
                    tsdf[idx] = (weight[idx] * tsdf[idx] + 1.0f * frk) / (weight[idx] + 1.0f);
                    weight[idx] = weight[idx] + 1.0f;
                }
            }
        }
    }
}

namespace {

/* Ray_Box_Intersection, voxel_traversal.cu:4-73 */
float slab_entry(bool& hit, F3 d, F3 lo, F3 hi, F3 o)
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
        hit = false;
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
        hit = false;
        return -1;
    }
    if (tz0 > t0) t0 = tz0;
    hit = true;
    return t0;
}

/* one ray of Voxel_Traversal, voxel_traversal.cu:86-423 */
void trace(const kfo_grid* g, int H, int W, int i, const float* depth, const float* Ki, const float* T,
           const float* tsdf, float* out6, int32_t* hit)
{
    const long HW = (long)H * W;
    for (int k = 0; k < 6; ++k) out6[k * HW + i] = 0.f;
    hit[i] = -1;
    const float D = depth[i];
    if (!(D != 0)) return;
    const int L = g->dims[0], Wd = g->dims[1], Hz = g->dims[2];
    const float vd = g->voxel_size;
    const F3 lo{(float)(g->start[0] * vd), (float)(g->start[1] * vd), (float)(g->start[2] * vd)};
    const F3 hi{(float)((g->start[0] + L) * vd), (float)((g->start[1] + Wd) * vd), (float)((g->start[2] + Hz) * vd)};

    const float X = (float)(i % W) + 1.0f, Y = (float)(i / W) + 1.0f;
    const F3 lam{Ki[0] * X + Ki[1] * Y + Ki[2] * 1.f, Ki[3] * X + Ki[4] * Y + Ki[5] * 1.f,
                 Ki[6] * X + Ki[7] * Y + Ki[8] * 1.f};
    const float lnorm = std::sqrt(lam.x * lam.x + lam.y * lam.y + lam.z * lam.z);
    /* start the ray truncated_distance before the measurement, :99-106 */
    const F3 sl{((lnorm * D - g->truncated_distance) / lnorm) * lam.x,
                ((lnorm * D - g->truncated_distance) / lnorm) * lam.y,
                ((lnorm * D - g->truncated_distance) / lnorm) * lam.z};
    const F3 org{T[0] * sl.x + T[1] * sl.y + T[2] * sl.z + T[3] * 1.f, T[4] * sl.x + T[5] * sl.y + T[6] * sl.z + T[7] * 1.f,
                 T[8] * sl.x + T[9] * sl.y + T[10] * sl.z + T[11] * 1.f};
    const F3 cam{T[3], T[7], T[11]};
    const F3 lg{T[0] * lam.x + T[1] * lam.y + T[2] * lam.z + T[3] * 1.f, T[4] * lam.x + T[5] * lam.y + T[6] * lam.z + T[7] * 1.f,
                T[8] * lam.x + T[9] * lam.y + T[10] * lam.z + T[11] * 1.f};
    const F3 dir = normalized(F3{lg.x - cam.x, lg.y - cam.y, lg.z - cam.z});

    bool inside = false;
    float tmin = slab_entry(inside, dir, lo, hi, org);
    if (!inside) return;
    if (tmin < 0) tmin = 0;
    const F3 s{org.x + tmin * dir.x, org.y + tmin * dir.y, org.z + tmin * dir.z};
    const F3 box{hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    int ix = (int)std::floor(((s.x - lo.x) / box.x) * L) + 1;
    int iy = (int)std::floor(((s.y - lo.y) / box.y) * Wd) + 1;
    int iz = (int)std::floor(((s.z - lo.z) / box.z) * Hz) + 1;
    /* never-assigned axis records: pinned to 0 (the reference leaves them uninitialised) */
    int XY = 0, XZ = 0, YX = 0, YZ = 0, ZX = 0, ZY = 0;
    if (ix == L + 1) ix = ix - 1;
    if (iy == Wd + 1) iy = iy - 1;
    if (iz == Hz + 1) iz = iz - 1;

    float tvx, tvy, tvz, sx, sy, sz;
    if (dir.x >= 0) { tvx = (float)(ix) / L; sx = 1; } else { tvx = (float)(ix - 1) / L; sx = -1; }
    if (dir.y >= 0) { tvy = (float)(iy) / Wd; sy = 1; } else { tvy = (float)(iy - 1) / Wd; sy = -1; }
    if (dir.z >= 0) { tvz = (float)(iz) / Hz; sz = 1; } else { tvz = (float)(iz - 1) / Hz; sz = -1; }
    const F3 vmax{lo.x + tvx * box.x, lo.y + tvy * box.y, lo.z + tvz * box.z};
    F3 tm{tmin + ((vmax.x - s.x) / dir.x), tmin + ((vmax.y - s.y) / dir.y), tmin + ((vmax.z - s.z) / dir.z)};
    const F3 dims{(float)L, (float)Wd, (float)Hz};
    const F3 td{vd / std::fabs(dir.x), vd / std::fabs(dir.y), vd / std::fabs(dir.z)};

    float prev = 0.0f;
    const long sx_ = (long)Wd * Hz, sy_ = Hz;
    long vi = (ix - 1) * sx_ + (iy - 1) * sy_ + (iz - 1);
    while (ix < (dims.x - 1) && ix > 0 && iy < (dims.y - 1) && iy > 0 && iz < (dims.z - 1) && iz > 0) {
        const float cur = tsdf[vi];
        if (std::isnan(cur) && prev < 0.f) break;
        if (cur < 0.f && std::isnan(prev)) break;
        if (cur > 0.f && prev < 0.f) break;
        if (cur < 0.f && prev > 0.f) {
            const int xn = (ix - 1) - 1, xp = (ix - 1) + 1;
            const int yn = (iy - 1) - 1, yp = (iy - 1) + 1;
            const int zn = (iz - 1) - 1, zp = (iz - 1) + 1;
            /* :233-282 -- note the recorded indices are range-checked against the
             * dimension of the axis that was stepped, as in the reference */
            if (xn >= L || xn < 0 || xp >= L || xp < 0) break;
            if ((XY - 1) >= L || (XY - 1) < 0 || (XZ - 1) >= L || (XZ - 1) < 0) break;
            if (yn >= Wd || yn < 0 || yp >= Wd || yp < 0) break;
            if ((YX - 1) >= Wd || (YX - 1) < 0 || (YZ - 1) >= Wd || (YZ - 1) < 0) break;
            if (zn >= Hz || zn < 0 || zp >= Hz || zp < 0) break;
            if ((ZX - 1) >= Hz || (ZX - 1) < 0 || (ZY - 1) >= Hz || (ZY - 1) < 0) break;
            const long x_np = xn * sx_ + (XY - 1) * sy_ + XZ - 1;
            const long x_pp = xp * sx_ + (XY - 1) * sy_ + XZ - 1;
            const long y_np = (YX - 1) * sx_ + yn * sy_ + YZ - 1;
            const long y_pp = (YX - 1) * sx_ + yp * sy_ + YZ - 1;
            const long z_np = (ZX - 1) * sx_ + (ZY - 1) * sy_ + zn;
            const long z_pp = (ZX - 1) * sx_ + (ZY - 1) * sy_ + zp;
            const long x_nn = (ix - 2) * sx_ + (iy - 1) * sy_ + (iz - 1);
            const long x_pn = (ix)*sx_ + (iy - 1) * sy_ + (iz - 1);
            const long y_nn = (ix - 1) * sx_ + (iy - 2) * sy_ + (iz - 1);
            const long y_pn = (ix - 1) * sx_ + (iy)*sy_ + (iz - 1);
            const long z_nn = (ix - 1) * sx_ + (iy - 1) * sy_ + (iz - 2);
            const long z_pn = (ix - 1) * sx_ + (iy - 1) * sy_ + (iz);
            if (std::isnan(tsdf[x_np]) || std::isnan(tsdf[x_pp]) || std::isnan(tsdf[y_np]) || std::isnan(tsdf[y_pp]) ||
                std::isnan(tsdf[z_np]) || std::isnan(tsdf[z_pp]) || std::isnan(tsdf[vi]))
                break;
            if (std::isnan(tsdf[x_nn]) || std::isnan(tsdf[x_pn]) || std::isnan(tsdf[y_nn]) || std::isnan(tsdf[y_pn]) ||
                std::isnan(tsdf[z_nn]) || std::isnan(tsdf[z_pn]))
                break;
            F3 sp, nr;
            /* per-axis linear zero crossing from the neighbour recorded at the last step
             * along that axis, :318-349 (coordinates from the voxel-centre formula) */
            if (dir.x > 0)
                sp.x = centre(xn, g->start[0], vd) + vd * (std::fabs(tsdf[x_np]) / (std::fabs(tsdf[x_np] - tsdf[vi])));
            else
                sp.x = centre(xp, g->start[0], vd) - vd * (std::fabs(tsdf[x_pp]) / (std::fabs(tsdf[x_pp] - tsdf[vi])));
            if (dir.y > 0)
                sp.y = centre(yn, g->start[1], vd) + vd * (std::fabs(tsdf[y_np]) / (std::fabs(tsdf[y_np] - tsdf[vi])));
            else
                sp.y = centre(yp, g->start[1], vd) - vd * (std::fabs(tsdf[y_pp]) / (std::fabs(tsdf[y_pp] - tsdf[vi])));
            if (dir.z > 0)
                sp.z = centre(zn, g->start[2], vd) + vd * (std::fabs(tsdf[z_np]) / (std::fabs(tsdf[z_np] - tsdf[vi])));
            else
                sp.z = centre(zp, g->start[2], vd) - vd * (std::fabs(tsdf[z_pp]) / (std::fabs(tsdf[z_pp] - tsdf[vi])));
            nr.x = (tsdf[x_pn] - tsdf[x_nn]) / 2.0f;
            nr.y = (tsdf[y_pn] - tsdf[y_nn]) / 2.0f;
            nr.z = (tsdf[z_pn] - tsdf[z_nn]) / 2.0f;
            const F3 va = normalized(F3{cam.x - sp.x, cam.y - sp.y, cam.z - sp.z});
            F3 vb = normalized(nr);
            const float ct = va.x * vb.x + va.y * vb.y + va.z * vb.z;
            if (kfo_raycast_flip(ct)) vb = F3{-vb.x, -vb.y, -vb.z};
            out6[0 * HW + i] = sp.x;
            out6[1 * HW + i] = sp.y;
            out6[2 * HW + i] = sp.z;
            out6[3 * HW + i] = vb.x;
            out6[4 * HW + i] = vb.y;
            out6[5 * HW + i] = vb.z;
            hit[i] = (int32_t)vi;
            break;
        }
        prev = cur;
        /* Amanatides-Woo step, :384-417 */
        if (tm.x < tm.y) {
            if (tm.x < tm.z) {
                ix = ix + sx; XY = iy; XZ = iz; tm.x = tm.x + td.x;
            } else {
                iz = iz + sz; ZX = ix; ZY = iy; tm.z = tm.z + td.z;
            }
        } else {
            if (tm.y < tm.z) {
                iy = iy + sy; YX = ix; YZ = iz; tm.y = tm.y + td.y;
            } else {
                iz = iz + sz; ZX = ix; ZY = iy; tm.z = tm.z + td.z;
            }
        }
        vi = (ix - 1) * sx_ + (iy - 1) * sy_ + (iz - 1);
    }
}

}  // namespace

void kfo_raycast(const kfo_grid* g, int H, int W, const float* depth, const float* Ki, const float* T,
                 const float* tsdf, float* out6, int32_t* hit)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < H * W; ++i) trace(g, H, W, i, depth, Ki, T, tsdf, out6, hit);
}

namespace {

/* per-pixel ICP row (sensor_pose_estimation.cu:20-131): returns true and fills the
 * 6 + 36 products when the pixel is a correspondence */
bool icp_terms(int H, int W, int i, const float* K, const float* F, const float* T, const float* cur6,
               const uint8_t* mask, const float* pred6, int32_t* pidx, float* t42)
{
    const long HW = (long)H * W;
    const float vx = cur6[0 * HW + i], vy = cur6[1 * HW + i], vz = cur6[2 * HW + i];
    *pidx = -1;
    if (!(vz != 0 && mask[i] != 0)) return false;
    const F3 c = xform_point(F, F3{vx, vy, vz});
    /* the reference projects through K although the parameter is named
     * dev_inv_cam_intrinsic (launch at :353 passes dev_cam_intrinsic) */
    const F3 p = mul3(K, c);
    const int u = (int)std::round(p.x / p.z);
    const int v = (int)std::round(p.y / p.z);
    if (!(u > 0 && u <= W && v > 0 && v <= H)) return false;
    const F3 g = xform_point(T, F3{vx, vy, vz});
    const int j = (v - 1) * W + (u - 1);
    const float qx = pred6[0 * HW + j], qy = pred6[1 * HW + j], qz = pred6[2 * HW + j];
    const float mx = pred6[3 * HW + j], my = pred6[4 * HW + j], mz = pred6[5 * HW + j];
    const F3 dd{g.x - qx, g.y - qy, g.z - qz};
    const float dist = std::sqrt(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
    if (!(dist <= 20.0f && dist >= 0.0f)) return false;
    const float nx = cur6[3 * HW + i], ny = cur6[4 * HW + i], nz = cur6[5 * HW + i];
    const F3 un = normalized(F3{T[0] * nx + T[1] * ny + T[2] * nz, T[4] * nx + T[5] * ny + T[6] * nz,
                                T[8] * nx + T[9] * ny + T[10] * nz});
    const F3 va = normalized(F3{mx, my, mz});
    const float ct = un.x * va.x + un.y * va.y + un.z * va.z;
    const float angle = kfo_icp_angle_deg(ct);
    if (!(angle <= 30.0f && angle >= 0.0f)) return false;
    float a[6];
    a[0] = g.z * my + (-g.y * mz);
    a[1] = -g.z * mx + (g.x * mz);
    a[2] = g.y * mx + (-g.x * my);
    a[3] = mx;
    a[4] = my;
    a[5] = mz;
    const float b = mx * (qx - g.x) + my * (qy - g.y) + mz * (qz - g.z);
    for (int r = 0; r < 6; ++r) t42[r] = a[r] * b;
    for (int r = 0; r < 6; ++r)
        for (int s = 0; s < 6; ++s) t42[6 + r * 6 + s] = a[r] * a[s];
    *pidx = j;
    return true;
}

}  // namespace

int kfo_icp_associate(int H, int W, const float* K, const float* F, const float* T, const float* cur6,
                      const uint8_t* mask, const float* pred6, int32_t* pair, float* sums42)
{
    const int n = H * W;
    const int nblocks = (n + 63) / 64;
    /* per 64-pixel block: tree reduction with strides 32..1 (Sum_Array, :225-245) */
    std::vector<float> partial((size_t)nblocks * 42);
    int ncorr = 0;
#pragma omp parallel for schedule(static) reduction(+ : ncorr)
    for (int b = 0; b < nblocks; ++b) {
        float sh[64][42];
        for (int t = 0; t < 64; ++t) {
            const int i = b * 64 + t;
            int32_t pidx = -1;
            for (int k = 0; k < 42; ++k) sh[t][k] = 0.f;
            if (i < n && icp_terms(H, W, i, K, F, T, cur6, mask, pred6, &pidx, sh[t])) ++ncorr;
            if (i < n && pair) pair[i] = pidx;
        }
        for (int s = 32; s > 0; s >>= 1)
            for (int t = 0; t < s; ++t)
                for (int k = 0; k < 42; ++k) sh[t][k] += sh[t + s][k];
        for (int k = 0; k < 42; ++k) partial[(size_t)b * 42 + k] = sh[0][k];
    }
    /* serial host sum over the block partials, :363-387 */
    for (int k = 0; k < 42; ++k) {
        float s = 0.0f;
        for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * 42 + k];
        sums42[k] = s;
    }
    return ncorr;
}

void kfo_icp_terms(int H, int W, const float* K, const float* F, const float* T, const float* cur6,
                   const uint8_t* mask, const float* pred6, float* terms42)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H * W; ++i) {
        int32_t pidx = -1;
        float t[42] = {};
        icp_terms(H, W, i, K, F, T, cur6, mask, pred6, &pidx, t);
        for (int k = 0; k < 42; ++k) terms42[(size_t)i * 42 + k] = t[k];
    }
}

namespace {

/* the ICP iterations of sensor_pose_estimation.cu:339-429 from a given T_prev^-1 (the
 * frame start's, :256), updating R in place */
void pose_iterations(int H, int W, const float* K, const float* Tprev_inv, float* R, const float* cur6,
                     const uint8_t* mask, const float* pred6, int iters, int log0, float* sums_log, float* pose_log,
                     int32_t* ncorr_log, int32_t* chol_ok_log)
{
    float F[16];
    for (int it = 0; it < iters; ++it) {
        ocv_matmul4(Tprev_inv, R, F);
        float s42[42];
        const int nc = kfo_icp_associate(H, W, K, F, R, cur6, mask, pred6, nullptr, s42);
        const int q = log0 + it;
        if (sums_log) std::memcpy(sums_log + q * 42, s42, sizeof(s42));
        float A[36], x[6];
        for (int k = 0; k < 36; ++k) A[k] = s42[6 + k];
        for (int k = 0; k < 6; ++k) x[k] = s42[k];
        /* return value ignored by the reference: a failed factorisation leaves b as is */
        const int ok = ocv_cholesky6(A, x);
        /* small-angle increment, :406-425; x = (beta, gamma, alpha, tx, ty, tz) */
        const float inc[16] = {1.0f, x[2], -x[1], x[3], -x[2], 1.0f, x[0], x[4],
                               x[1], -x[0], 1.0f, x[5], 0.0f, 0.0f, 0.0f, 1.0f};
        ocv_matmul4(inc, R, R);
        if (pose_log) std::memcpy(pose_log + q * 16, R, sizeof(float) * 16);
        if (ncorr_log) ncorr_log[q] = nc;
        if (chol_ok_log) chol_ok_log[q] = ok;
    }
}

}  // namespace

void kfo_estimate_pose(int H, int W, const float* K, float* T, const float* cur6, const uint8_t* mask,
                       const float* pred6, int iters, float* sums_log, float* pose_log, int32_t* ncorr_log,
                       int32_t* chol_ok_log)
{
    float Tprev_inv[16], R[16];
    ocv_inv4(T, Tprev_inv);
    std::memcpy(R, T, sizeof(R));
    pose_iterations(H, W, K, Tprev_inv, R, cur6, mask, pred6, iters, 0, sums_log, pose_log, ncorr_log, chol_ok_log);
    std::memcpy(T, R, sizeof(R));
}

/* ICP pyramid (not in the reference): coarse (i, j) averages the nonzero depths of the
 * fine 2x2 block, scan order (2i,2j), (2i,2j+1), (2i+1,2j), (2i+1,2j+1), that lie within
 * band of the block's first nonzero depth; 0 where the block has none */
void kfo_pyramid_depth(int Hf, int Wf, const float* fine, float band, float* coarse)
{
    const int Hc = Hf / 2, Wc = Wf / 2;
    for (int r = 0; r < Hc; ++r)
        for (int c = 0; c < Wc; ++c) {
            const float d[4] = {fine[(2 * r) * Wf + 2 * c], fine[(2 * r) * Wf + 2 * c + 1],
                                fine[(2 * r + 1) * Wf + 2 * c], fine[(2 * r + 1) * Wf + 2 * c + 1]};
            float ref = 0.f;
            for (int k = 0; k < 4 && ref == 0.f; ++k) ref = d[k];
            float sum = 0.f;
            int n = 0;
            for (int k = 0; k < 4; ++k)
                if (d[k] != 0.f && std::fabs(d[k] - ref) <= band) {
                    sum = sum + d[k];
                    ++n;
                }
            coarse[r * Wc + c] = n ? sum / (float)n : 0.f;
        }
}

/* the intrinsics of pyramid level l: focal lengths / 2^l, 1-based principal point
 * (c - 1/2) / 2^l + 1/2 */
void kfo_level_intrinsics(const float* K, int l, float* Kl)
{
    const float s = 1.0f / (float)(1 << l);
    const float k[9] = {K[0] * s, 0.0f, (K[2] - 0.5f) * s + 0.5f, 0.0f, K[4] * s, (K[5] - 0.5f) * s + 0.5f,
                        0.0f, 0.0f, 1.0f};
    std::memcpy(Kl, k, sizeof(k));
}

/* bilateral_filtering.cu:3-47 */
void kfo_bilateral(int H, int W, const float* depth, const float* spatial, int r, float sigma_r, float* out)
{
    const int kl = 2 * r + 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H * W; ++i) {
        out[i] = 0.f;
        const int y0 = i / W, x0 = i % W;
        if (!(y0 >= r && y0 <= H - 1 - r && x0 >= r && x0 <= W - 1 - r)) continue;
        const float c = depth[i];
        float w[64 * 64];
        float sum = 0.f;
        for (int y = y0 - r; y <= y0 + r; ++y)
            for (int x = x0 - r; x <= x0 + r; ++x) {
                float t = depth[y * W + x] - c;
                t = std::exp(-(t * t) / (2 * sigma_r * sigma_r));
                const float wt = spatial[(y - y0 + r) * kl + (x - x0 + r)] * t + 0.000000001f;
                w[(y - y0 + r) * kl + (x - x0 + r)] = wt;
                sum = sum + wt;
            }
        float acc = 0.f;
        for (int y = y0 - r; y <= y0 + r; ++y)
            for (int x = x0 - r; x <= x0 + r; ++x)
                acc = acc + (w[(y - y0 + r) * kl + (x - x0 + r)] / sum) * depth[y * W + x];
        out[i] = acc;
    }
}

/* ---------------- KinfuPipeline frame loop ---------------- */

struct kfo_pipeline {
    int H, W;
    float min_depth, max_depth;
    kfo_grid g;
    float K[9], Ki[9], T[16];
    int icp_iters;
    int levels = 1, level_iters[3] = {10, 0, 0};
    float band = 90.f;
    int bilateral = 0, bil_r = 3;
    float sigma_r = 30.f;
    std::vector<float> spatial, filtered;
    std::vector<float> tsdf, weight, depth, cur6, pred6;
    std::vector<uint8_t> mask;
    std::vector<int32_t> hit;
};

kfo_pipeline* kfo_create(int H, int W, float min_depth, float max_depth, const kfo_grid* g, const float* K,
                         int icp_iters)
{
    kfo_pipeline* p = new kfo_pipeline;
    p->H = H;
    p->W = W;
    p->min_depth = min_depth;
    p->max_depth = max_depth;
    p->g = *g;
    std::memcpy(p->K, K, sizeof(p->K));
    ocv_inv3(p->K, p->Ki);
    for (int i = 0; i < 16; ++i) p->T[i] = (i % 5 == 0) ? 1.f : 0.f;
    p->icp_iters = icp_iters;
    const size_t n = (size_t)g->dims[0] * g->dims[1] * g->dims[2];
    /* kinfu_pipeline.cpp:61-64: volume starts as NaN */
    p->tsdf.assign(n, NAN);
    p->weight.assign(n, NAN);
    p->depth.assign((size_t)H * W, 0.f);
    p->cur6.assign((size_t)6 * H * W, 0.f);
    p->pred6.assign((size_t)6 * H * W, 0.f);
    p->mask.assign((size_t)H * W, 0);
    p->hit.assign((size_t)H * W, -1);
    return p;
}

void kfo_destroy(kfo_pipeline* p) { delete p; }

void kfo_initial(kfo_pipeline* p, const uint16_t* raw)
{
    const int H = p->H, W = p->W;
    kfo_depth_ingest(raw, H * W, p->min_depth, p->max_depth, p->depth.data());
    float Ti[16];
    ocv_inv4(p->T, Ti);
    kfo_integrate(&p->g, H, W, p->depth.data(), p->K, p->Ki, p->T, Ti, p->tsdf.data(), p->weight.data(), 1);
    kfo_raycast(&p->g, H, W, p->depth.data(), p->Ki, p->T, p->tsdf.data(), p->pred6.data(), p->hit.data());
}

void kfo_set_pyramid(kfo_pipeline* p, int levels, const int* iters, float band)
{
    p->levels = levels < 1 ? 1 : (levels > 3 ? 3 : levels);
    for (int l = 0; l < 3; ++l) p->level_iters[l] = l < p->levels ? iters[l] : 0;
    p->band = band;
}

/* the bilateral stage at the reference's commented-out call site
 * (kinfu_pipeline.cpp:141-145): its spatial kernel as SystemUtility::CreateSpatialKernel
 * (system_utility.cpp:94-113) */
void kfo_set_bilateral(kfo_pipeline* p, int enable, int radius, float sigma_d, float sigma_r)
{
    p->bilateral = enable != 0;
    p->bil_r = radius;
    p->sigma_r = sigma_r;
    const int kl = 2 * radius + 1;
    p->spatial.assign((size_t)kl * kl, 0.f);
    for (int y = -radius; y <= radius; ++y)
        for (int x = -radius; x <= radius; ++x) {
            const float e = -((float)(x * x) + (float)(y * y)) / (2 * sigma_d * sigma_d);
            p->spatial[(y + radius) * kl + (x + radius)] = (float)std::exp((double)e);
        }
}

static void incoming(kfo_pipeline* p, const uint16_t* raw, const float* filtered_in);

void kfo_incoming(kfo_pipeline* p, const uint16_t* raw) { incoming(p, raw, nullptr); }

void kfo_incoming_filtered(kfo_pipeline* p, const uint16_t* raw, const float* filtered)
{
    incoming(p, raw, filtered);
}

static void incoming(kfo_pipeline* p, const uint16_t* raw, const float* filtered_in)
{
    const int H = p->H, W = p->W;
    const long HW = (long)H * W;
    kfo_depth_ingest(raw, H * W, p->min_depth, p->max_depth, p->depth.data());
    float* c = p->cur6.data();
    kfo_vertex_normal(H, W, p->depth.data(), p->Ki, c, c + HW, c + 3 * HW, c + 4 * HW, c + 5 * HW, p->mask.data());
    if (p->bilateral) {
        /* the filtered depth is fed forward as if written over depth_image_next (the
         * reference's commented-out call writes bilateral_output, which nothing reads):
         * ICP reads it as the vertices' z, integration and the ray cast as the depth */
        p->filtered.assign(HW, 0.f);
        if (filtered_in)
            std::memcpy(p->filtered.data(), filtered_in, sizeof(float) * HW);
        else
            kfo_bilateral(H, W, p->depth.data(), p->spatial.data(), p->bil_r, p->sigma_r, p->filtered.data());
        p->depth = p->filtered;
    }
    std::memcpy(c + 2 * HW, p->depth.data(), sizeof(float) * HW);
    if (p->levels == 1) {
        kfo_estimate_pose(H, W, p->K, p->T, c, p->mask.data(), p->pred6.data(), p->icp_iters, nullptr, nullptr,
                          nullptr, nullptr);
    } else {
        /* per level: depth, K, vertex/normal map (cur6 layout) and the previous
         * prediction subsampled at (2i, 2j) */
        std::vector<float> depth[3], cur[3], pred[3];
        std::vector<uint8_t> mask[3];
        float Kl[3][9];
        depth[0] = p->depth;
        cur[0] = p->cur6;
        pred[0] = p->pred6;
        mask[0] = p->mask;
        std::memcpy(Kl[0], p->K, sizeof(Kl[0]));
        for (int l = 1; l < p->levels; ++l) {
            const int Hf = H >> (l - 1), Wf = W >> (l - 1), Hc = H >> l, Wc = W >> l;
            const long n = (long)Hc * Wc, nf = (long)Hf * Wf;
            depth[l].assign(n, 0.f);
            kfo_pyramid_depth(Hf, Wf, depth[l - 1].data(), p->band, depth[l].data());
            kfo_level_intrinsics(p->K, l, Kl[l]);
            float Kil[9];
            ocv_inv3(Kl[l], Kil);
            cur[l].assign(6 * n, 0.f);
            mask[l].assign(n, 0);
            float* q = cur[l].data();
            kfo_vertex_normal(Hc, Wc, depth[l].data(), Kil, q, q + n, q + 3 * n, q + 4 * n, q + 5 * n, mask[l].data());
            std::memcpy(q + 2 * n, depth[l].data(), sizeof(float) * n);
            pred[l].assign(6 * n, 0.f);
            for (int k = 0; k < 6; ++k)
                for (long i = 0; i < n; ++i)
                    pred[l][k * n + i] = pred[l - 1][k * nf + (2 * (i / Wc)) * Wf + 2 * (i % Wc)];
        }
        float Tprev_inv[16];
        ocv_inv4(p->T, Tprev_inv);
        for (int l = p->levels - 1; l >= 0; --l)
            pose_iterations(H >> l, W >> l, Kl[l], Tprev_inv, p->T, cur[l].data(), mask[l].data(), pred[l].data(),
                            p->level_iters[l], 0, nullptr, nullptr, nullptr, nullptr);
    }
    float Ti[16];
    ocv_inv4(p->T, Ti);
    kfo_integrate(&p->g, H, W, p->depth.data(), p->K, p->Ki, p->T, Ti, p->tsdf.data(), p->weight.data(), 0);
    kfo_raycast(&p->g, H, W, p->depth.data(), p->Ki, p->T, p->tsdf.data(), p->pred6.data(), p->hit.data());
}

void kfo_get_pose(const kfo_pipeline* p, float* T) { std::memcpy(T, p->T, sizeof(p->T)); }
void kfo_set_pose(kfo_pipeline* p, const float* T) { std::memcpy(p->T, T, sizeof(p->T)); }

void kfo_get_prediction(const kfo_pipeline* p, float* out6, int32_t* hit)
{
    if (out6) std::memcpy(out6, p->pred6.data(), sizeof(float) * p->pred6.size());
    if (hit) std::memcpy(hit, p->hit.data(), sizeof(int32_t) * p->hit.size());
}

void kfo_get_volume(const kfo_pipeline* p, float* tsdf, float* weight)
{
    if (tsdf) std::memcpy(tsdf, p->tsdf.data(), sizeof(float) * p->tsdf.size());
    if (weight) std::memcpy(weight, p->weight.data(), sizeof(float) * p->weight.size());
}

void kfo_get_depth(const kfo_pipeline* p, float* depth)
{
    std::memcpy(depth, p->depth.data(), sizeof(float) * p->depth.size());
}

void kfo_get_vertex_map(const kfo_pipeline* p, float* cur6, uint8_t* mask)
{
    if (cur6) std::memcpy(cur6, p->cur6.data(), sizeof(float) * p->cur6.size());
    if (mask) std::memcpy(mask, p->mask.data(), p->mask.size());
}

}  // extern "C"
