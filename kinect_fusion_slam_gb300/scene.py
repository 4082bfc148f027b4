"""Seeded synthetic depth sequences: an analytic room seen by a Kinect v1 camera.

Stand-in for the reference's recorded scan (its data/dep0024..0300.dat frames): an
axis-aligned room whose outer box is the reference volume (3.6 x 3.6 x 3.0 m, walls
0.1 m thick, so the inner faces lie 0.1 m inside the grid), six spheres (radius
0.1-0.4 m) and four boxes (edges 0.2-0.6 m) at seeded uniform positions in front of
the first camera, a seeded smooth random-walk trajectory (1-2 cm and 0.5-1 degree per
frame), and 640x480 uint16 millimetre depth from an exact ray cast of the analytic
scene with the Kinect v1 axial noise model sigma(z) = 0.0012 + 0.0019 (z - 0.4)^2 m and
2 % random dropout.

Everything is computed with +, -, *, / and sqrt on float64 from a counter-based
integer hash, so a sequence depends only on its seed, not on the platform's libm.
Units are millimetres and the first pose is the identity, as in the reference
(kinfu_pipeline.cpp:6-65).  Intrinsics are returned in the reference's 1-based
convention (principal point + 1), which is what the pipeline consumes.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    x = x.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        x ^= x >> np.uint64(30)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
    return x


def uniform(seed: int, stream: int, counter: np.ndarray | int) -> np.ndarray:
    """Uniform [0, 1) doubles keyed by (seed, stream, counter)."""
    c = np.asarray(counter, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = _mix(np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + np.uint64(stream) * np.uint64(0xD1B54A32D192ED03))
        x = _mix(c * np.uint64(0x9E3779B97F4A7C15) + key)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def gaussian(seed: int, stream: int, counter: np.ndarray | int) -> np.ndarray:
    """Approximately standard normal (Irwin-Hall sum of 12 uniforms, minus 6)."""
    c = np.asarray(counter, dtype=np.uint64) * np.uint64(12)
    acc = np.zeros(np.shape(c), np.float64)
    for k in range(12):
        acc = acc + uniform(seed, stream, c + np.uint64(k))
    return acc - 6.0


@dataclass(frozen=True)
class Camera:
    """Kinect v1 pinhole model; cx, cy are 0-based (pixel centres at integers)."""

    width: int = 640
    height: int = 480
    fx: float = 525.0
    fy: float = 525.0
    cx: float = 319.5
    cy: float = 239.5

    def K_reference(self) -> np.ndarray:
        """3x3 intrinsic matrix in the reference's 1-based pixel convention."""
        return np.array([[self.fx, 0.0, self.cx + 1.0], [0.0, self.fy, self.cy + 1.0], [0.0, 0.0, 1.0]], np.float32)

    def scaled(self, s: float) -> "Camera":
        return Camera(int(self.width * s), int(self.height * s), self.fx * s, self.fy * s,
                      (self.cx + 0.5) * s - 0.5, (self.cy + 0.5) * s - 0.5)


@dataclass(frozen=True)
class GridConfig:
    dims: tuple = (360, 360, 300)
    voxel_size: float = 10.0
    truncated_distance: float = 300.0
    sdf_minimum: float = -30.0
    sdf_maximum: float = 300.0
    # reference volume [-2000, 1600] x [-2000, 1600] x [-1200, 1800] mm
    origin_mm: tuple = (-2000.0, -2000.0, -1200.0)

    @property
    def start(self) -> tuple:
        """Integer voxel coordinate of voxel (0,0,0) (kinfu_pipeline.h:43-45)."""
        return tuple(int(round(o / self.voxel_size)) for o in self.origin_mm)

    @property
    def nvox(self) -> int:
        return int(self.dims[0]) * int(self.dims[1]) * int(self.dims[2])


@dataclass(frozen=True)
class SceneConfig:
    name: str
    grid: GridConfig
    frames: int
    camera: Camera = field(default_factory=Camera)
    seed: int = 1234
    icp_levels: tuple = (10,)
    min_depth: float = 300.0
    max_depth: float = 2000.0
    noise: bool = True
    dropout: float = 0.02


def config(name: str, **overrides) -> SceneConfig:
    """The five workloads: c0 small, c1 default, c2 precision, c3 differentiation
    grid, c4 batching (one of its scenes; see ``batch_configs``)."""
    presets = {
        "c0": SceneConfig("c0", GridConfig((180, 180, 150), 20.0), 20, seed=1000),
        "c1": SceneConfig("c1", GridConfig((360, 360, 300), 10.0), 300, seed=1001),
        "c2": SceneConfig("c2", GridConfig((512, 512, 430), 7.0), 300, seed=1002),
        "c3": SceneConfig("c3", GridConfig((256, 256, 256), 10.0, origin_mm=(-1280.0, -1280.0, -280.0)), 64,
                          seed=1003),
        "c4": SceneConfig("c4", GridConfig((128, 128, 128), 20.0, origin_mm=(-1280.0, -1280.0, -400.0)), 100,
                          seed=1004),
    }
    cfg = presets[name]
    if overrides:
        d = dict(cfg.__dict__)
        d.update(overrides)
        cfg = SceneConfig(**d)
    return cfg


def batch_configs(n: int = 16, seed: int = 2000) -> list[SceneConfig]:
    """Uneven scenes for the batching workload: grids 128^3 @ 2 cm, 256^3 @ 1.5 cm and
    384x384x320 @ 1 cm; depth 320x240 or 640x480; 100 frames each."""
    grids = [GridConfig((128, 128, 128), 20.0, origin_mm=(-1280.0, -1280.0, -400.0)),
             GridConfig((256, 256, 256), 15.0, origin_mm=(-1920.0, -1920.0, -900.0)),
             GridConfig((384, 384, 320), 10.0, origin_mm=(-1920.0, -1920.0, -1200.0))]
    out = []
    for i in range(n):
        g = grids[i % 3]
        cam = Camera() if (i // 3) % 2 == 0 else Camera().scaled(0.5)
        out.append(SceneConfig(f"c4_{i}", g, 100, camera=cam, seed=seed + i))
    return out


# ----------------------------------------------------------------------------- scene
@dataclass
class Scene:
    room_lo: np.ndarray
    room_hi: np.ndarray
    spheres: np.ndarray  # (n, 4) centre xyz, radius
    boxes: np.ndarray  # (n, 6) lo xyz, hi xyz


def make_scene(cfg: SceneConfig) -> Scene:
    g = cfg.grid
    lo = np.array(g.origin_mm, np.float64)
    hi = lo + np.array(g.dims, np.float64) * g.voxel_size
    wall = 100.0
    room_lo, room_hi = lo + wall, hi - wall
    seed = cfg.seed
    # objects in the half of the room in front of the first camera (z > 0)
    spheres, boxes = [], []
    k = 0
    while len(spheres) < 6:
        u = uniform(seed, 1, np.arange(k * 4, k * 4 + 4, dtype=np.uint64))
        k += 1
        r = 100.0 + 300.0 * u[3]
        c_lo = np.array([room_lo[0] + r, room_lo[1] + r, max(0.0, room_lo[2]) + r])
        c_hi = room_hi - r
        c = c_lo + (c_hi - c_lo) * u[:3]
        if np.sqrt(np.sum(c * c)) < r + 700.0:
            continue
        spheres.append([c[0], c[1], c[2], r])
    k = 0
    while len(boxes) < 4:
        u = uniform(seed, 2, np.arange(k * 6, k * 6 + 6, dtype=np.uint64))
        k += 1
        e = 200.0 + 400.0 * u[3:6]
        b_lo = np.array([room_lo[0], room_lo[1], max(0.0, room_lo[2])])
        b_hi = room_hi - e
        p = b_lo + (b_hi - b_lo) * u[:3]
        centre = p + e / 2
        if np.sqrt(np.sum(centre * centre)) < np.sqrt(np.sum(e * e)) / 2 + 700.0:
            continue
        boxes.append([*p, *(p + e)])
    return Scene(room_lo, room_hi, np.array(spheres), np.array(boxes))


# ------------------------------------------------------------------------ trajectory
def _quat_to_R(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _unit(v: np.ndarray) -> np.ndarray:
    return v / np.sqrt(np.sum(v * v))


def trajectory(cfg: SceneConfig) -> np.ndarray:
    """(frames, 4, 4) float64 camera-to-world poses in mm; poses[0] = identity.

    Each frame moves 10-20 mm along a smoothly drifting direction (pulled back
    towards the start when more than 0.4 m away) and turns 0.5-1 degree about a
    smoothly drifting axis (pulled back towards the initial heading)."""
    seed = cfg.seed
    n = cfg.frames
    poses = np.zeros((n, 4, 4))
    R = np.eye(3)
    p = np.zeros(3)
    d = _unit(gaussian(seed, 3, np.arange(3, dtype=np.uint64)) + np.array([0.0, 0.0, 0.5]))
    w = _unit(gaussian(seed, 4, np.arange(3, dtype=np.uint64)))
    deg = np.pi / 180.0
    for k in range(n):
        poses[k, :3, :3] = R
        poses[k, :3, 3] = p
        poses[k, 3, 3] = 1.0
        gk = gaussian(seed, 5, np.arange(6 * k + 6, 6 * k + 12, dtype=np.uint64))
        uk = uniform(seed, 6, np.arange(2 * k, 2 * k + 2, dtype=np.uint64))
        dist = np.sqrt(np.sum(p * p))
        pull = -p / dist * min(1.0, max(0.0, dist - 400.0) / 200.0) if dist > 0 else np.zeros(3)
        d = _unit(d + 0.25 * gk[:3] + pull)
        fwd = R[:, 2]
        w = _unit(w + 0.25 * gk[3:] + 0.5 * np.cross(fwd, np.array([0.0, 0.0, 1.0])))
        step = 10.0 + 10.0 * uk[0]
        ang = (0.5 + 0.5 * uk[1]) * deg
        p = p + step * d
        # q = normalise(1, (ang/2) w): a rotation by 2 atan(ang/2) ~ ang (within 3e-5 relative)
        q = np.array([1.0, *(0.5 * ang * w)])
        q = q / np.sqrt(np.sum(q * q))
        R = _quat_to_R(q) @ R
    return poses


# ---------------------------------------------------------------------------- render
def render_depth_mm(cfg: SceneConfig, scene: Scene, pose: np.ndarray, frame: int) -> np.ndarray:
    """Exact analytic ray cast -> Kinect-noised uint16 depth (mm), (H, W)."""
    cam = cfg.camera
    H, W = cam.height, cam.width
    cols = np.arange(W, dtype=np.float64)
    rows = np.arange(H, dtype=np.float64)
    dx = np.broadcast_to((cols - cam.cx) / cam.fx, (H, W)).ravel()
    dy = np.broadcast_to(((rows - cam.cy) / cam.fy)[:, None], (H, W)).ravel()
    dcam = np.stack([dx, dy, np.ones_like(dx)], 1)  # camera z component 1 -> t is the depth
    R, o = pose[:3, :3], pose[:3, 3]
    d = dcam @ R.T
    t = np.full(dx.shape, np.inf)
    # room: the ray leaves the inner box through the nearest wall
    with np.errstate(divide="ignore", invalid="ignore"):
        for a in range(3):
            bound = np.where(d[:, a] > 0, scene.room_hi[a], scene.room_lo[a])
            ta = (bound - o[a]) / d[:, a]
            ta = np.where(d[:, a] != 0, ta, np.inf)
            t = np.minimum(t, np.where(ta > 0, ta, np.inf))
        for cx, cy, cz, r in scene.spheres:
            oc = o - np.array([cx, cy, cz])
            a2 = np.sum(d * d, 1)
            b = np.sum(d * oc, 1)
            c = np.sum(oc * oc) - r * r
            disc = b * b - a2 * c
            ts = (-b - np.sqrt(np.maximum(disc, 0.0))) / a2
            t = np.where((disc >= 0) & (ts > 0) & (ts < t), ts, t)
        for bx in scene.boxes:
            t0 = np.full(dx.shape, -np.inf)
            t1 = np.full(dx.shape, np.inf)
            for a in range(3):
                inv = 1.0 / d[:, a]
                ta = (bx[a] - o[a]) * inv
                tb = (bx[a + 3] - o[a]) * inv
                t0 = np.maximum(t0, np.minimum(ta, tb))
                t1 = np.minimum(t1, np.maximum(ta, tb))
            t = np.where((t1 >= t0) & (t0 > 0) & (t0 < t), t0, t)
    z = t / 1000.0  # metres
    idx = np.arange(H * W, dtype=np.uint64) + np.uint64(frame) * np.uint64(H * W)
    if cfg.noise:
        sigma = 0.0012 + 0.0019 * (z - 0.4) * (z - 0.4)
        z = z + sigma * gaussian(cfg.seed, 7, idx)
    mm = np.floor(z * 1000.0 + 0.5)
    mm = np.where(np.isfinite(mm), mm, 0.0)
    mm = np.clip(mm, 0.0, 65535.0)
    if cfg.dropout > 0:
        mm = np.where(uniform(cfg.seed, 8, idx) < cfg.dropout, 0.0, mm)
    return mm.astype(np.uint16).reshape(H, W)


@dataclass
class Sequence:
    cfg: SceneConfig
    scene: Scene
    poses: np.ndarray  # (frames, 4, 4) float64 ground truth, mm
    K: np.ndarray  # reference-convention intrinsics

    def depth(self, k: int) -> np.ndarray:
        return render_depth_mm(self.cfg, self.scene, self.poses[k], k)

    def depths(self, n: int | None = None) -> np.ndarray:
        n = self.cfg.frames if n is None else n
        return np.stack([self.depth(k) for k in range(n)])


def sequence(cfg: SceneConfig | str, frames: int | None = None) -> Sequence:
    if isinstance(cfg, str):
        cfg = config(cfg)
    if frames is not None:
        cfg = SceneConfig(**{**cfg.__dict__, "frames": frames})
    return Sequence(cfg, make_scene(cfg), trajectory(cfg), cfg.camera.K_reference())


def _render_task(task):
    cfg, k = task
    seq = sequence(cfg)
    return render_depth_mm(cfg, seq.scene, seq.poses[k], k)


def render_sequences(cfgs: list[SceneConfig], frames: int, processes: int | None = None) -> list[np.ndarray]:
    """The first `frames` depth frames of each scene, (frames, H, W) uint16 per scene,
    rendered by a pool of spawned processes (the renderer is CPU numpy; spawned workers
    start fresh interpreters, so a caller that has already initialised CUDA is safe).
    Identical to Sequence.depths, frame for frame."""
    import multiprocessing as mp
    import os

    cfgs = [SceneConfig(**{**c.__dict__, "frames": max(frames, c.frames)}) for c in cfgs]
    tasks = [(c, k) for c in cfgs for k in range(frames)]
    n = processes or min(len(tasks), os.cpu_count() or 1)
    if n <= 1:
        out = [_render_task(t) for t in tasks]
    else:
        with mp.get_context("spawn").Pool(n) as pool:
            out = pool.map(_render_task, tasks, chunksize=max(1, len(tasks) // (4 * n)))
    return [np.stack(out[i * frames:(i + 1) * frames]) for i in range(len(cfgs))]
