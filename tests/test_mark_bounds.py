"""Integration lists only the voxel boxes that the marking pass (integrate_mark_kernel and
integrate_list_kernel in csrc/kf_tsdf.cu) proves can hold an updated voxel.  The GPU
tests hold the kernels to the oracle bit for bit on chosen cameras and poses; this CPU
test checks the bounds themselves on many random ones.  The marking pass's formulas are
restated here in float32 numpy (depth-band slabs of every 8x8 depth tile, the grid's far
corner, the mirrored slabs behind the camera, the near-camera boxes, the rigid-pose
fallback), and every voxel the oracle updates must fall in a listed box: cameras with
focal lengths of 12 to 900 px and principal points off the image, grids up to 320 m
from the origin, rotation blocks up to 1.5e-4 from orthonormal, and depths with holes,
near samples, negative, NaN, 1e30 and infinite values."""
import dataclasses

import numpy as np
import pytest

from conftest import grid_spec

f32 = np.float32
K_SLAB, K_MAX_SLABS, K_NEAR_Z, K_NEAR_R, K_RIGID_TOL = f32(80), 512, f32(100), f32(250), f32(2e-4)
BOX_X, BOX_Y, BOX_Z, TILE = 32, 8, 8, 8


def depth_band_eps(K, W, H):
    fx, fy, cx, cy = f32(K[0, 0]), f32(K[1, 1]), f32(K[0, 2]), f32(K[1, 2])
    a = (max(cx, f32(W) + f32(1) - cx) + f32(1)) / fx
    b = (max(cy, f32(H) + f32(1) - cy) + f32(1)) / fy
    dx, dy = f32(0.5) / fx, f32(0.5) / fy
    return f32(2) * (f32(2) * a * dx + dx * dx + f32(2) * b * dy + dy * dy) + f32(1e-4)


def ray_norm_max(Ki, W, H):
    m = max(np.linalg.norm(Ki.astype(np.float64) @ np.array([u, v, 1.0])) for u in (1, W) for v in (1, H))
    return f32(m * 1.01 + 1e-3)


def rigid_error(T):
    R = T[:3, :3].astype(np.float32)
    return float(np.max(np.abs(R.T @ R - np.eye(3, dtype=np.float32))))


def listed_boxes(gs, K, Ki, T, depth):
    """The boxes (z, y, x) the marking and list passes put on the list."""
    H, W = depth.shape
    dims, start, vd = gs.dims, gs.start, f32(gs.voxel_size)
    nb = (-(-dims[2] // BOX_Z), -(-dims[1] // BOX_Y), -(-dims[0] // BOX_X))
    mark = np.zeros(nb, bool)
    fx, fy, cx, cy = f32(K[0, 0]), f32(K[1, 1]), f32(K[0, 2]), f32(K[1, 2])
    deps, lam = depth_band_eps(K, W, H), ray_norm_max(Ki, W, H)
    t = T[:3, 3]
    tmax = f32(np.max(np.abs(t)))
    mark_all = rigid_error(T) > K_RIGID_TOL
    mark_near = False
    hi_band, lo_band = f32(max(gs.sdf_maximum, 0)), f32(min(gs.sdf_minimum, 0))
    eps_t = f32(2.0 ** -18) * (tmax + f32(4) * lam + f32(1))
    abs_t = f32(2.0 ** -19) * tmax + f32(1)
    ext = f32(max(max(abs(s), abs(s + d)) for s, d in zip(start, dims))) * vd
    far2 = f32(0)
    for a in range(3):
        d = max(abs((f32(start[a]) + f32(0.5)) * vd - t[a]), abs((f32(start[a] + dims[a]) - f32(0.5)) * vd - t[a]))
        far2 += d * d
    z_far = np.sqrt(far2) * f32(1.01) + f32(2) * vd + f32(1)
    g_lo = np.array([(f32(s) - 1) * vd for s in start], np.float32)
    g_hi = np.array([(f32(s + d) + 1) * vd for s, d in zip(start, dims)], np.float32)
    ad = np.abs(depth.astype(np.float32))
    for ty in range(-(-H // TILE)):
        for tx in range(-(-W // TILE)):
            blk = ad[ty * TILE:(ty + 1) * TILE, tx * TILE:(tx + 1) * TILE]
            v = blk[(blk != 0) & ~np.isnan(blk)]
            if v.size == 0:
                continue
            dmin, dmax = f32(v.min()), f32(v.max())
            with np.errstate(all="ignore"):
                z_a = (dmin * (f32(1) - eps_t) - hi_band - f32(2) * abs_t) / ((f32(1) + deps) * (f32(1) + eps_t)) \
                    * f32(0.999) - f32(1)
                den_b = (f32(1) - deps) * (f32(1) - eps_t)
                z_b = ((dmax * (f32(1) + eps_t) - lo_band + f32(2) * abs_t) / den_b * f32(1.001) + f32(1)) \
                    if den_b > 0.5 else f32(np.inf)
            if z_a < K_NEAR_Z:
                mark_near = True
            if np.isnan(z_far):
                continue
            z_lo = max(z_a, K_NEAR_Z) if not np.isnan(z_a) else K_NEAR_Z
            z_hi = min(z_b, z_far)
            if not z_hi > z_lo:
                continue
            span = z_hi - z_lo
            if not span < 1e30:
                mark_all = True
                continue
            slab = max(K_SLAB, span * f32(1.0 / K_MAX_SLABS))
            nslab = min(K_MAX_SLABS, int(np.ceil(span / slab)))
            err_l = f32(2.0 ** -19) * f32(4) * (ext + tmax)
            mpx = f32(1) + (max(fx, fy) + max(abs(cx), abs(cy)) + f32(max(W, H)) + f32(10)) * err_l / z_lo + f32(1e-3)
            u_a, v_a = f32(tx * TILE) + f32(0.5), f32(ty * TILE) + f32(0.5)
            rx0, rx1 = (u_a - mpx - cx) / fx, (u_a + f32(8) + mpx - cx) / fx
            ry0, ry1 = (v_a - mpx - cy) / fy, (v_a + f32(8) + mpx - cy) / fy
            wr = [T[:3, 0] * (rx1 if c & 1 else rx0) + T[:3, 1] * (ry1 if c & 2 else ry0) + T[:3, 2] for c in range(4)]
            rmax = max(abs(rx0), abs(rx1), abs(ry0), abs(ry1))
            ca_x, ca_y = (cy - cx) / fx, (cx - cy) / fy
            s_min = f32(1) + min(ca_x * rx0, ca_x * rx1) + min(ca_y * ry0, ca_y * ry1)
            ca_n = f32(1) + abs(ca_x) + abs(ca_y)
            s_margin = (f32(2.0 ** -18) * (ca_n + f32(2) * tmax) + f32(4) * K_RIGID_TOL * ca_n) * lam + f32(1e-3)
            nside = 1 if s_min > s_margin else 2
            for k in range(nside * nslab):
                ks, sgn = (k, f32(1)) if k < nslab else (k - nslab, f32(-1))
                za = z_lo + f32(ks) * slab
                zb = z_hi if ks == nslab - 1 else min(z_lo + f32(ks + 1) * slab, z_hi)
                pts = np.array([wr[c & 3] * (sgn * (zb if c & 4 else za)) + t for c in range(8)], np.float32)
                e = f32(2.0 ** -17) * ((f32(2) * rmax + f32(1)) * f32(2) * zb + tmax) + f32(1)
                lo, hi = pts.min(0) - e, pts.max(0) + e
                if not (np.all(lo <= g_hi) and np.all(hi >= g_lo)):
                    continue
                lo, hi = np.maximum(lo, g_lo), np.minimum(hi, g_hi)
                i0 = [max(0, int(np.floor((lo[a] - f32(0.5) * vd) / vd)) - start[a]) for a in range(3)]
                i1 = [min(dims[a] - 1, int(np.ceil((hi[a] - f32(0.5) * vd) / vd)) - start[a]) for a in range(3)]
                if any(i0[a] > i1[a] for a in range(3)):
                    continue
                mark[i0[2] // BOX_Z:i1[2] // BOX_Z + 1, i0[1] // BOX_Y:i1[1] // BOX_Y + 1,
                     i0[0] // BOX_X:i1[0] // BOX_X + 1] = True
    if mark_all:
        mark[:] = True
    elif mark_near:
        near_r = max(K_NEAR_R, K_NEAR_Z * lam) + f32(2) * vd
        ok = np.ones(nb, bool)
        for a, (n, ax) in enumerate(((BOX_X, 2), (BOX_Y, 1), (BOX_Z, 0))):
            i0 = np.arange(nb[ax]) * n
            lo = (f32(1) * (i0 + start[a]) + f32(0.5)) * vd
            hi = (f32(1) * (i0 + n - 1 + start[a]) + f32(0.5)) * vd
            hit = (hi >= t[a] - near_r) & (lo <= t[a] + near_r)
            shape = [1, 1, 1]
            shape[ax] = nb[ax]
            ok &= hit.reshape(shape)
        mark |= ok
    return mark


def _rot(rng, ang):
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    Kx = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    return np.eye(3) + np.sin(ang) * Kx + (1 - np.cos(ang)) * Kx @ Kx


def _trial(oracle, seed):
    from kinect_fusion_slam_gb300 import scene

    rng = np.random.default_rng(seed)
    W, H = [(64, 48), (96, 64), (160, 120)][rng.integers(3)]
    f = float(np.exp(rng.uniform(np.log(12), np.log(900))))
    K = np.array([[f * rng.uniform(0.7, 1.3), 0, rng.uniform(-0.2, 1.2) * W + 1],
                  [0, f * rng.uniform(0.7, 1.3), rng.uniform(-0.2, 1.2) * H + 1], [0, 0, 1]], np.float32)
    vd = float(rng.choice([10.0, 20.0, 37.0]))
    dims = tuple(int(v) for v in rng.integers(20, 90, 3))
    off = int(rng.choice([0, 0, 0, 2500, 16000, -9000]))
    start = tuple(int(-d // 2) + off for d in dims)
    gs = dataclasses.replace(grid_spec(scene.GridConfig(dims, vd)), start=start)
    Ki = oracle.inv3(K)
    centre = (np.array(start) + np.array(dims) / 2) * vd
    cam = centre + rng.normal(size=3) * np.array(dims) * vd * rng.uniform(0, 0.8)
    R = _rot(rng, rng.uniform(0, np.pi))
    if rng.random() < 0.6:  # towards the grid centre, or directly away from it
        zc = centre - cam
        zc /= np.linalg.norm(zc) + 1e-9
        if rng.random() < 0.3:
            zc = -zc
        xc = np.cross(rng.normal(size=3), zc)
        xc /= np.linalg.norm(xc)
        R = np.stack([xc, np.cross(zc, xc), zc], 1) @ _rot(rng, rng.uniform(0, 0.3))
    if rng.random() < 0.35:  # drifted off orthonormal, inside the tolerance
        R = R @ (np.eye(3) + rng.uniform(-5e-5, 5e-5, (3, 3)))
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, cam
    T = T.astype(np.float32)
    near_frac = 0.05 if rng.random() < 0.4 else 0.0
    base = max(400.0 if near_frac else 1200.0, np.linalg.norm(centre - cam) * rng.uniform(0.3, 1.5))
    yy, xx = np.mgrid[0:H, 0:W]
    depth = (base + rng.uniform(0, 0.5) * base * np.sin(xx / rng.uniform(3, 20)) *
             np.cos(yy / rng.uniform(3, 20))).astype(np.float32)
    for val, frac in [(0.0, 0.2), (None, near_frac), (-1.0, 0.01), (np.nan, 0.01), (np.inf, 0.005), (1e30, 0.005)]:
        m = rng.random((H, W)) < frac
        if val is None:
            depth[m] = rng.uniform(10, 300, int(m.sum()))
        elif val == -1.0:
            depth[m] *= -1
        else:
            depth[m] = val
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=True)
    upd = np.flatnonzero(~np.isnan(wo))  # z-fastest: ((x * dy) + y) * dz + z
    x, y, z = upd // (dims[1] * dims[2]), (upd // dims[2]) % dims[1], upd % dims[2]
    mark = listed_boxes(gs, K, Ki, T, depth)
    return int(np.count_nonzero(~mark[z // BOX_Z, y // BOX_Y, x // BOX_X])), upd.size


def test_marks_cover_every_updated_voxel(oracle):
    updated = 0
    for seed in range(80):
        m, u = _trial(oracle, seed)
        assert m == 0, f"seed {seed}: {m} updated voxels outside the listed boxes"
        updated += u
    assert updated > 100_000


def test_marks_cover_wide_angle_near_voxels(oracle):
    """A 30 px focal length on 160 x 120 with depths of 50-150 mm: voxels updated closer
    than the first slab lie up to ~350 mm from the camera, beyond the fixed 250 mm, and
    the near radius grows with the ray norm to bound them (here the boxes' size and the
    per-axis test leave the fixed radius enough slack as well)."""
    from kinect_fusion_slam_gb300 import scene

    g = scene.GridConfig((180, 180, 150), 20.0)
    gs = grid_spec(g)
    W, H = 160, 120
    K = np.array([[30.0, 0.0, W / 2 + 0.5], [0.0, 30.0, H / 2 + 0.5], [0.0, 0.0, 1.0]], np.float32)
    Ki = oracle.inv3(K)
    rng = np.random.default_rng(17)
    for yaw, t in [(0.3, (200.0, -150.0, -300.0)), (-0.5, (-400.0, 300.0, 100.0)), (1.2, (0.0, 0.0, 500.0))]:
        T = np.eye(4)
        T[:3, :3] = _rot(np.random.default_rng(int(yaw * 10) + 5), yaw)
        T[:3, 3] = t
        T = T.astype(np.float32)
        yy, xx = np.mgrid[0:H, 0:W]
        depth = (400.0 + 300.0 * np.sin(xx / 9.0) * np.cos(yy / 7.0)).astype(np.float32)
        near = rng.random((H, W)) < 0.1
        depth[near] = rng.uniform(50.0, 150.0, int(near.sum())).astype(np.float32)
        to = np.full(gs.nvox, np.nan, np.float32)
        wo = np.full(gs.nvox, np.nan, np.float32)
        oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=True)
        upd = np.flatnonzero(~np.isnan(wo))
        x, y, z = upd // (g.dims[1] * g.dims[2]), (upd // g.dims[2]) % g.dims[1], upd % g.dims[2]
        mark = listed_boxes(gs, K, Ki, T, depth)
        assert upd.size > 10_000
        assert not np.any(~mark[z // BOX_Z, y // BOX_Y, x // BOX_X])
