/*
 * TEST INFRASTRUCTURE -- the FP64 oracle (see kf_oracle.h).  Never part of the product.
 *
 * The reference's per-frame algorithm (PoChang007/Kinect_Fusion_SLAM) with every
 * floating-point quantity in double: depth, vertex and normal maps, the TSDF values and
 * weights, the ray cast, the ICP association, its normal equations (summed in double)
 * and a plain double Cholesky solve, and the pose, which is never rounded to float.
 * The algorithm keeps every convention of the float restatement in kf_oracle.cpp --
 * 1-based pixels, the swapped principal point of the in-front test, the per-axis
 * zero-crossing interpolation and the never-assigned axis records pinned to 0, the
 * uncapped weight -- so the only difference from the reference is precision.  The
 * precision form of the GPU pipeline (FP16 TSDF, compensated FP32 sums, FP64 solve) is
 * measured by its TSDF, prediction and trajectory error against this run.
 */
#include "kf_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct D3 {
    double x, y, z;
};

D3 xf(const double* m, D3 p)
{
    return D3{m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}

D3 m3(const double* m, D3 p)
{
    return D3{m[0] * p.x + m[1] * p.y + m[2] * p.z, m[3] * p.x + m[4] * p.y + m[5] * p.z,
              m[6] * p.x + m[7] * p.y + m[8] * p.z};
}

D3 unit(D3 v)
{
    const double r = 1.0 / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return D3{v.x * r, v.y * r, v.z * r};
}

double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

double centre64(int index, int start, double vd) { return (double)(index + start) * vd + vd / 2.0; }

void inv3_64(const double* m, double* o)
{
    const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    const double r = 1.0 / det;
    o[0] = c00 * r;
    o[1] = (m[2] * m[7] - m[1] * m[8]) * r;
    o[2] = (m[1] * m[5] - m[2] * m[4]) * r;
    o[3] = c01 * r;
    o[4] = (m[0] * m[8] - m[2] * m[6]) * r;
    o[5] = (m[2] * m[3] - m[0] * m[5]) * r;
    o[6] = c02 * r;
    o[7] = (m[1] * m[6] - m[0] * m[7]) * r;
    o[8] = (m[0] * m[4] - m[1] * m[3]) * r;
}

// Gauss-Jordan with partial pivoting; false when singular
bool inv4_64(const double* src, double* out)
{
    double a[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) a[i][j] = j < 4 ? src[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0) return false;
        if (p != c)
            for (int j = 0; j < 8; ++j) std::swap(a[p][j], a[c][j]);
        const double inv = 1.0 / a[c][c];
        for (int j = 0; j < 8; ++j) a[c][j] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double f = a[r][c];
            for (int j = 0; j < 8; ++j) a[r][j] -= f * a[c][j];
        }
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) out[i * 4 + j] = a[i][j + 4];
    return true;
}

void mul4_64(const double* a, const double* b, double* out)
{
    double r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r[i * 4 + j] = a[i * 4] * b[j] + a[i * 4 + 1] * b[4 + j] + a[i * 4 + 2] * b[8 + j] + a[i * 4 + 3] * b[12 + j];
    std::memcpy(out, r, sizeof(r));
}

// A x = b for symmetric positive definite A (6x6 row-major, full); false otherwise
bool chol6_64(const double* A_in, double* b)
{
    double L[36];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = A_in[i * 6 + j];
            for (int k = 0; k < j; ++k) s -= L[i * 6 + k] * L[j * 6 + k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                L[i * 6 + i] = std::sqrt(s);
            } else {
                L[i * 6 + j] = s / L[j * 6 + j];
            }
        }
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[i * 6 + k] * b[k];
        b[i] = s / L[i * 6 + i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = b[i];
        for (int k = i + 1; k < 6; ++k) s -= L[k * 6 + i] * b[k];
        b[i] = s / L[i * 6 + i];
    }
    return true;
}

const double kPi = 3.14159265358979323846;

}  // namespace

struct kfo64_pipeline {
    int H, W;
    double min_depth, max_depth;
    kfo_grid g;
    double K[9], Ki[9], T[16];
    int icp_iters;
    std::vector<double> tsdf, weight, depth, vx, vy, nx, ny, nz, pred6;
    std::vector<uint8_t> mask;
};

namespace {

void ingest(kfo64_pipeline* p, const uint16_t* raw)
{
    for (int i = 0; i < p->H * p->W; ++i) {
        const double d = (double)raw[i];
        p->depth[i] = (d >= p->min_depth && d <= p->max_depth) ? d : 0.0;
    }
}

// raw_vertices.cu:3-51 in double
void vertex_normal(kfo64_pipeline* p)
{
    const int H = p->H, W = p->W;
    const double* Ki = p->Ki;
    const double* depth = p->depth.data();
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H * W; ++i) {
        p->vx[i] = p->vy[i] = p->nx[i] = p->ny[i] = p->nz[i] = 0.0;
        p->mask[i] = 0;
        const int row = i / W, col = i % W;
        if (!(depth[i] != 0 && row != H - 1 && col != W - 1)) continue;
        p->mask[i] = 1;
        const int down = (row + 1) * W + col, right = row * W + col + 1;
        if (!(depth[down] != 0 && depth[right] != 0)) continue;
        const double d = depth[i], dd = depth[down], dr = depth[right];
        const double X = col + 1, Y = row + 1;
        const double px = d * (Ki[0] * X + Ki[1] * Y + Ki[2]), py = d * (Ki[3] * X + Ki[4] * Y + Ki[5]);
        const double dx = dd * (Ki[0] * X + Ki[1] * (Y + 1) + Ki[2]), dy = dd * (Ki[3] * X + Ki[4] * (Y + 1) + Ki[5]);
        const double rx = dr * (Ki[0] * (X + 1) + Ki[1] * Y + Ki[2]), ry = dr * (Ki[3] * (X + 1) + Ki[4] * Y + Ki[5]);
        const double n0 = (dy - py) * (dr - d) - (dd - d) * (ry - py);
        const double n1 = (dd - d) * (rx - px) - (dx - px) * (dr - d);
        const double n2 = (dx - px) * (ry - py) - (dy - py) * (rx - px);
        const double len = std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
        p->vx[i] = px;
        p->vy[i] = py;
        p->nx[i] = n0 / len;
        p->ny[i] = n1 / len;
        p->nz[i] = n2 / len;
    }
}

// projective_tsdf.cu:5-140 in double
void integrate(kfo64_pipeline* p, bool first)
{
    const kfo_grid* g = &p->g;
    const int H = p->H, W = p->W, DX = g->dims[0], DY = g->dims[1], DZ = g->dims[2];
    const double vd = g->voxel_size, trunc = g->truncated_distance, smin = g->sdf_minimum, smax = g->sdf_maximum;
    const double *K = p->K, *Ki = p->Ki, *T = p->T;
    double Ti[16];
    inv4_64(T, Ti);
    const D3 cam{T[3], T[7], T[11]};
    const D3 ca = m3(Ki, D3{K[5], K[2], 1.0});
    const D3 ga = xf(T, ca), gb = xf(T, D3{2 * ca.x, 2 * ca.y, 2 * ca.z});
    const D3 axis{gb.x - ga.x, gb.y - ga.y, gb.z - ga.z};
    const double* depth = p->depth.data();
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < DX; ++ix) {
        const double cx = centre64(ix, g->start[0], vd);
        for (int iy = 0; iy < DY; ++iy) {
            const double cy = centre64(iy, g->start[1], vd);
            for (int iz = 0; iz < DZ; ++iz) {
                const long idx = ((long)ix * DY + iy) * DZ + iz;
                const D3 c{cx, cy, centre64(iz, g->start[2], vd)};
                const D3 q = m3(K, xf(Ti, c));
                const int u = (int)std::round(q.x / q.z), v = (int)std::round(q.y / q.z);
                if (!(u > 0 && u <= W && v > 0 && v <= H)) continue;
                const double D = depth[(v - 1) * W + (u - 1)];
                if (!(D != 0)) continue;
                const D3 lam = m3(Ki, D3{(double)u, (double)v, 1.0});
                const D3 dir{T[0] * lam.x + T[1] * lam.y + T[2] * lam.z, T[4] * lam.x + T[5] * lam.y + T[6] * lam.z,
                             T[8] * lam.x + T[9] * lam.y + T[10] * lam.z};
                const double mag = std::sqrt(dot(dir, dir));
                const D3 td{c.x - cam.x, c.y - cam.y, c.z - cam.z};
                if (!(dot(axis, td) > 0)) continue;
                const D3 pt = xf(T, D3{D * lam.x, D * lam.y, D * lam.z});
                const D3 rel{pt.x - cam.x, pt.y - cam.y, pt.z - cam.z};
                double frk = std::sqrt(dot(rel, rel)) / mag - std::sqrt(dot(td, td)) / mag;
                const bool ahead = frk > 0 && frk <= smax, behind = frk <= 0 && frk >= smin;
                if (!ahead && !behind) continue;
                frk = ahead ? std::fmin(1.0, frk / trunc) : std::fmax(-1.0, frk / trunc);
                double& t = p->tsdf[idx];
                double& w = p->weight[idx];
                if (first) {
                    t = frk;
                    w = 1.0;
                } else {
                    if (std::isnan(t)) t = 0.0;
                    if (std::isnan(w)) w = 0.0;
                    t = (w * t + frk) / (w + 1.0);
                    w = w + 1.0;
                }
            }
        }
    }
}

double slab64(bool& hit, D3 d, D3 lo, D3 hi, D3 o)
{
    double t0, t1, ty0, ty1, tz0, tz1;
    if (d.x >= 0) { t0 = (lo.x - o.x) / d.x; t1 = (hi.x - o.x) / d.x; } else { t0 = (hi.x - o.x) / d.x; t1 = (lo.x - o.x) / d.x; }
    if (d.y >= 0) { ty0 = (lo.y - o.y) / d.y; ty1 = (hi.y - o.y) / d.y; } else { ty0 = (hi.y - o.y) / d.y; ty1 = (lo.y - o.y) / d.y; }
    if (t0 > ty1 || ty0 > t1) { hit = false; return -1; }
    if (ty0 > t0) t0 = ty0;
    if (ty1 < t1) t1 = ty1;
    if (d.z >= 0) { tz0 = (lo.z - o.z) / d.z; tz1 = (hi.z - o.z) / d.z; } else { tz0 = (hi.z - o.z) / d.z; tz1 = (lo.z - o.z) / d.z; }
    if (t0 > tz1 || tz0 > t1) { hit = false; return -1; }
    if (tz0 > t0) t0 = tz0;
    hit = true;
    return t0;
}

// one ray of voxel_traversal.cu:86-423 in double
void trace64(const kfo64_pipeline* p, int i, double* out6)
{
    const kfo_grid* g = &p->g;
    const long HW = (long)p->H * p->W;
    for (int k = 0; k < 6; ++k) out6[k * HW + i] = 0.0;
    const double D = p->depth[i];
    if (!(D != 0)) return;
    const int L = g->dims[0], Wd = g->dims[1], Hz = g->dims[2];
    const double vd = g->voxel_size;
    const double *Ki = p->Ki, *T = p->T;
    const double* tsdf = p->tsdf.data();
    const D3 lo{g->start[0] * vd, g->start[1] * vd, g->start[2] * vd};
    const D3 hi{(g->start[0] + L) * vd, (g->start[1] + Wd) * vd, (g->start[2] + Hz) * vd};
    const D3 lam = m3(Ki, D3{(double)(i % p->W) + 1.0, (double)(i / p->W) + 1.0, 1.0});
    const double ln = std::sqrt(dot(lam, lam));
    const double sc = (ln * D - g->truncated_distance) / ln;
    const D3 org = xf(T, D3{sc * lam.x, sc * lam.y, sc * lam.z});
    const D3 cam{T[3], T[7], T[11]};
    const D3 lg = xf(T, lam);
    const D3 dir = unit(D3{lg.x - cam.x, lg.y - cam.y, lg.z - cam.z});
    bool inside = false;
    double tmin = slab64(inside, dir, lo, hi, org);
    if (!inside) return;
    if (tmin < 0) tmin = 0;
    const D3 s{org.x + tmin * dir.x, org.y + tmin * dir.y, org.z + tmin * dir.z};
    const D3 box{hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    int ix = (int)std::floor(((s.x - lo.x) / box.x) * L) + 1;
    int iy = (int)std::floor(((s.y - lo.y) / box.y) * Wd) + 1;
    int iz = (int)std::floor(((s.z - lo.z) / box.z) * Hz) + 1;
    int XY = 0, XZ = 0, YX = 0, YZ = 0, ZX = 0, ZY = 0;
    if (ix == L + 1) --ix;
    if (iy == Wd + 1) --iy;
    if (iz == Hz + 1) --iz;
    double tvx, tvy, tvz;
    int sx, sy, sz;
    if (dir.x >= 0) { tvx = (double)ix / L; sx = 1; } else { tvx = (double)(ix - 1) / L; sx = -1; }
    if (dir.y >= 0) { tvy = (double)iy / Wd; sy = 1; } else { tvy = (double)(iy - 1) / Wd; sy = -1; }
    if (dir.z >= 0) { tvz = (double)iz / Hz; sz = 1; } else { tvz = (double)(iz - 1) / Hz; sz = -1; }
    D3 tm{tmin + (lo.x + tvx * box.x - s.x) / dir.x, tmin + (lo.y + tvy * box.y - s.y) / dir.y,
          tmin + (lo.z + tvz * box.z - s.z) / dir.z};
    const D3 tdl{vd / std::fabs(dir.x), vd / std::fabs(dir.y), vd / std::fabs(dir.z)};
    const long sxs = (long)Wd * Hz, sys = Hz;
    auto at = [&](long a, long b, long c) { return tsdf[a * sxs + b * sys + c]; };
    double prev = 0.0;
    while (ix < L - 1 && ix > 0 && iy < Wd - 1 && iy > 0 && iz < Hz - 1 && iz > 0) {
        const double cur = at(ix - 1, iy - 1, iz - 1);
        if (std::isnan(cur) && prev < 0) break;
        if (cur < 0 && std::isnan(prev)) break;
        if (cur > 0 && prev < 0) break;
        if (cur < 0 && prev > 0) {
            const int xn = ix - 2, xp = ix, yn = iy - 2, yp = iy, zn = iz - 2, zp = iz;
            if (xn >= L || xn < 0 || xp >= L || xp < 0) break;
            if (XY - 1 >= L || XY - 1 < 0 || XZ - 1 >= L || XZ - 1 < 0) break;
            if (yn >= Wd || yn < 0 || yp >= Wd || yp < 0) break;
            if (YX - 1 >= Wd || YX - 1 < 0 || YZ - 1 >= Wd || YZ - 1 < 0) break;
            if (zn >= Hz || zn < 0 || zp >= Hz || zp < 0) break;
            if (ZX - 1 >= Hz || ZX - 1 < 0 || ZY - 1 >= Hz || ZY - 1 < 0) break;
            const double x_np = at(xn, XY - 1, XZ - 1), x_pp = at(xp, XY - 1, XZ - 1);
            const double y_np = at(YX - 1, yn, YZ - 1), y_pp = at(YX - 1, yp, YZ - 1);
            const double z_np = at(ZX - 1, ZY - 1, zn), z_pp = at(ZX - 1, ZY - 1, zp);
            const double x_nn = at(ix - 2, iy - 1, iz - 1), x_pn = at(ix, iy - 1, iz - 1);
            const double y_nn = at(ix - 1, iy - 2, iz - 1), y_pn = at(ix - 1, iy, iz - 1);
            const double z_nn = at(ix - 1, iy - 1, iz - 2), z_pn = at(ix - 1, iy - 1, iz);
            if (std::isnan(x_np) || std::isnan(x_pp) || std::isnan(y_np) || std::isnan(y_pp) || std::isnan(z_np) ||
                std::isnan(z_pp) || std::isnan(cur))
                break;
            if (std::isnan(x_nn) || std::isnan(x_pn) || std::isnan(y_nn) || std::isnan(y_pn) || std::isnan(z_nn) ||
                std::isnan(z_pn))
                break;
            D3 sp;
            sp.x = dir.x > 0 ? centre64(xn, g->start[0], vd) + vd * (std::fabs(x_np) / std::fabs(x_np - cur))
                             : centre64(xp, g->start[0], vd) - vd * (std::fabs(x_pp) / std::fabs(x_pp - cur));
            sp.y = dir.y > 0 ? centre64(yn, g->start[1], vd) + vd * (std::fabs(y_np) / std::fabs(y_np - cur))
                             : centre64(yp, g->start[1], vd) - vd * (std::fabs(y_pp) / std::fabs(y_pp - cur));
            sp.z = dir.z > 0 ? centre64(zn, g->start[2], vd) + vd * (std::fabs(z_np) / std::fabs(z_np - cur))
                             : centre64(zp, g->start[2], vd) - vd * (std::fabs(z_pp) / std::fabs(z_pp - cur));
            const D3 va = unit(D3{cam.x - sp.x, cam.y - sp.y, cam.z - sp.z});
            D3 vb = unit(D3{(x_pn - x_nn) / 2.0, (y_pn - y_nn) / 2.0, (z_pn - z_nn) / 2.0});
            if (std::acos(dot(va, vb)) * (180.0 / kPi) > 90) vb = D3{-vb.x, -vb.y, -vb.z};
            const double o[6] = {sp.x, sp.y, sp.z, vb.x, vb.y, vb.z};
            for (int k = 0; k < 6; ++k) out6[k * HW + i] = o[k];
            break;
        }
        prev = cur;
        if (tm.x < tm.y) {
            if (tm.x < tm.z) { ix += sx; XY = iy; XZ = iz; tm.x += tdl.x; }
            else { iz += sz; ZX = ix; ZY = iy; tm.z += tdl.z; }
        } else {
            if (tm.y < tm.z) { iy += sy; YX = ix; YZ = iz; tm.y += tdl.y; }
            else { iz += sz; ZX = ix; ZY = iy; tm.z += tdl.z; }
        }
    }
}

void raycast(kfo64_pipeline* p)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < p->H * p->W; ++i) trace64(p, i, p->pred6.data());
}

// sensor_pose_estimation.cu:7-136 + :339-429 in double, with a double Cholesky solve
void estimate_pose(kfo64_pipeline* p)
{
    const int H = p->H, W = p->W;
    const long HW = (long)H * W;
    double Tprev_inv[16], F[16];
    inv4_64(p->T, Tprev_inv);
    const double* K = p->K;
    const double* pred = p->pred6.data();
    for (int it = 0; it < p->icp_iters; ++it) {
        mul4_64(Tprev_inv, p->T, F);
        const double* T = p->T;
        double sums[42] = {};
#pragma omp parallel
        {
            double loc[42] = {};
#pragma omp for schedule(static)
            for (int i = 0; i < H * W; ++i) {
                if (!(p->depth[i] != 0 && p->mask[i] != 0)) continue;
                const D3 v{p->vx[i], p->vy[i], p->depth[i]};
                const D3 q = m3(K, xf(F, v));
                const int u = (int)std::round(q.x / q.z), w = (int)std::round(q.y / q.z);
                if (!(u > 0 && u <= W && w > 0 && w <= H)) continue;
                const D3 gv = xf(T, v);
                const long j = (long)(w - 1) * W + (u - 1);
                const D3 sp{pred[j], pred[HW + j], pred[2 * HW + j]};
                const D3 m{pred[3 * HW + j], pred[4 * HW + j], pred[5 * HW + j]};
                const D3 dd{gv.x - sp.x, gv.y - sp.y, gv.z - sp.z};
                const double dist = std::sqrt(dot(dd, dd));
                if (!(dist <= 20.0 && dist >= 0.0)) continue;
                const D3 n{p->nx[i], p->ny[i], p->nz[i]};
                const D3 un = unit(D3{T[0] * n.x + T[1] * n.y + T[2] * n.z, T[4] * n.x + T[5] * n.y + T[6] * n.z,
                                      T[8] * n.x + T[9] * n.y + T[10] * n.z});
                const double angle = std::acos(dot(un, unit(m))) * (180.0 / kPi);
                if (!(angle <= 30.0 && angle >= 0.0)) continue;
                const double a[6] = {gv.z * m.y - gv.y * m.z, -gv.z * m.x + gv.x * m.z, gv.y * m.x - gv.x * m.y,
                                     m.x, m.y, m.z};
                const double b = m.x * (sp.x - gv.x) + m.y * (sp.y - gv.y) + m.z * (sp.z - gv.z);
                for (int r = 0; r < 6; ++r) loc[r] += a[r] * b;
                for (int r = 0; r < 6; ++r)
                    for (int c = 0; c < 6; ++c) loc[6 + r * 6 + c] += a[r] * a[c];
            }
#pragma omp critical
            for (int k = 0; k < 42; ++k) sums[k] += loc[k];
        }
        double x[6];
        for (int k = 0; k < 6; ++k) x[k] = sums[k];
        // the reference ignores a failed factorisation and applies b as it stands
        chol6_64(sums + 6, x);
        const double inc[16] = {1.0, x[2], -x[1], x[3], -x[2], 1.0, x[0], x[4], x[1], -x[0], 1.0, x[5], 0, 0, 0, 1.0};
        mul4_64(inc, p->T, p->T);
    }
}

}  // namespace

extern "C" {

kfo64_pipeline* kfo64_create(int H, int W, double min_depth, double max_depth, const kfo_grid* g, const double* K,
                             int icp_iters)
{
    kfo64_pipeline* p = new kfo64_pipeline;
    p->H = H;
    p->W = W;
    p->min_depth = min_depth;
    p->max_depth = max_depth;
    p->g = *g;
    std::memcpy(p->K, K, sizeof(p->K));
    inv3_64(p->K, p->Ki);
    for (int i = 0; i < 16; ++i) p->T[i] = (i % 5 == 0) ? 1.0 : 0.0;
    p->icp_iters = icp_iters;
    const size_t n = (size_t)g->dims[0] * g->dims[1] * g->dims[2], hw = (size_t)H * W;
    p->tsdf.assign(n, NAN);
    p->weight.assign(n, NAN);
    for (auto* v : {&p->depth, &p->vx, &p->vy, &p->nx, &p->ny, &p->nz}) v->assign(hw, 0.0);
    p->pred6.assign(6 * hw, 0.0);
    p->mask.assign(hw, 0);
    return p;
}

void kfo64_destroy(kfo64_pipeline* p) { delete p; }

void kfo64_initial(kfo64_pipeline* p, const uint16_t* raw)
{
    ingest(p, raw);
    integrate(p, true);
    raycast(p);
}

void kfo64_incoming(kfo64_pipeline* p, const uint16_t* raw)
{
    ingest(p, raw);
    vertex_normal(p);
    estimate_pose(p);
    integrate(p, false);
    raycast(p);
}

void kfo64_get_pose(const kfo64_pipeline* p, double* T) { std::memcpy(T, p->T, sizeof(p->T)); }

void kfo64_set_pose(kfo64_pipeline* p, const double* T) { std::memcpy(p->T, T, sizeof(p->T)); }

/* single stages at the current pose: ingest + integration of one frame, and the ray cast
 * of the current depth */
void kfo64_integrate_frame(kfo64_pipeline* p, const uint16_t* raw, int first)
{
    ingest(p, raw);
    integrate(p, first != 0);
}

void kfo64_raycast_frame(kfo64_pipeline* p) { raycast(p); }

void kfo64_get_prediction(const kfo64_pipeline* p, double* out6)
{
    std::memcpy(out6, p->pred6.data(), sizeof(double) * p->pred6.size());
}

void kfo64_get_volume(const kfo64_pipeline* p, float* tsdf, float* weight)
{
    for (size_t i = 0; i < p->tsdf.size(); ++i) {
        if (tsdf) tsdf[i] = (float)p->tsdf[i];
        if (weight) weight[i] = (float)p->weight[i];
    }
}

}  // extern "C"
