#!/usr/bin/env python
"""Frame-loop benchmark of the GB300 KinectFusion path.

One step = one IncomingFrameProcessing (vertex/normal map, single-level 10-iteration
ICP, TSDF integration, ray cast) on a 640x480 depth frame into the reference's
default 360x360x300 TSDF at 10 mm (workload c1).  Input: a seeded synthetic
sequence (analytic room, Kinect v1 noise model) of 48 frames, played forwards then
backwards; the pipeline starts over (reset + InitialProcessing) at the start of each
94-frame period, so a step is an InitialProcessing on 1 frame in 94.

  value   frames/s with the depth frames already in device memory (all ranks)
  e2e     frames/s through the C ABI with host buffers: each frame's uint16 depth is
          copied from pinned host memory and the pose read back to the host
  roofline   the dominant stage's algorithmic bytes per frame over its live time,
             against the measured copy bandwidth; DRAM traffic from the committed ncu
             launch lists (profiles/ncu_traffic.txt)
  cpu_baseline  the reference's kernel bodies on the host cores, a bounded sample
  clocks     SM clock and throttle reasons sampled during the timed region
  stages_ms  per-stage device time of a few frames (CUDA events inside the graph)
  ate        trajectory error against the FP64 oracle's trajectory (golden file)
  synced_fp64  per-frame pose error of a step taken from the FP64 oracle's state (golden
             file), the measure behind the precision form's <= 1 mm bar
  fp32_form, precision_c2, pyramid_c1, batching_c4, differentiation_c3: the other
             forms and workloads

--impl reference times the reference's own kernel bodies compiled for the host CPU
(oracle/_ref, or the oracle restatement where that could not be built) on the same
workload, with every host core.

Multi-GPU (--gpus N under torchrun): independent replicas, one scene per GPU, no
collective on the data path; the timed region is bracketed by barriers and the max
over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "frames/s (640x480, 360x360x300 TSDF) FP16-TSDF vs FP32 form at <=1 mm ATE"
UNIQUE_FRAMES = 48


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--config", default="c1")
    p.add_argument("--form", choices=["both", "precision", "plain"], default="both",
                   help="precision: FP16 TSDF, compensated one-pass sums, FP64 solve; plain: the bit-exact FP32 form")
    p.add_argument("--profile-frames", type=int, default=30, help="frames with per-stage CUDA events")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-ate", action="store_true", help="skip the trajectory comparison with the FP64 oracle")
    p.add_argument("--no-extra-forms", action="store_true", help="skip the batching (c4) and differentiation (c3) runs")
    p.add_argument("--batch-frames", type=int, default=100, help="frames per scene of the batching run (c4)")
    return p.parse_args(argv)


def pingpong(n_unique: int, n: int) -> list[int]:
    """0, 1, ..., n_unique-1, n_unique-2, ..., 1, 0, 1, ... (a continuous trajectory)."""
    period = max(1, 2 * (n_unique - 1))
    out = []
    for k in range(n):
        r = k % period if n_unique > 1 else 0
        out.append(r if r < n_unique else period - r)
    return out


def restarts(n_unique: int, n: int) -> list[bool]:
    """True where the pipeline starts over (reset + InitialProcessing): frame 0 of every
    forward-and-back period.  The reference's tracker drifts on this sequence (its
    projective TSDF gradients follow the viewing rays, so point-to-plane ICP constrains
    mostly depth) and loses lock after several periods; starting every period afresh
    keeps the per-frame work that of a tracked sequence for any step count."""
    period = max(1, 2 * (n_unique - 1))
    return [k % period == 0 for k in range(n)]


class Dist:
    """torch.distributed plumbing for replicas: barrier and max over ranks only."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            backend = "nccl" if os.environ.get("KF_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
            dist.init_process_group(backend=backend)
            self.pg = dist
            self.backend = backend

    def barrier(self):
        if self.pg:
            if self.backend == "nccl":
                import torch

                self.pg.barrier(device_ids=[self.local_rank])
            else:
                self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = f"cuda:{self.local_rank}" if self.backend == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.out.flush()
        self.out.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.out.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(args):
    from kinect_fusion_slam_gb300 import scene

    cfg = scene.config(args.config)
    return cfg


def config_desc(cfg, args) -> dict:
    g = cfg.grid
    return {
        "workload": (f"{cfg.name}: {cfg.camera.width}x{cfg.camera.height} uint16 depth, "
                     f"{g.dims[0]}x{g.dims[1]}x{g.dims[2]} TSDF @ {g.voxel_size:g} mm, single-level ICP x10, "
                     "integration + ray cast per frame"),
        "frames_unique": UNIQUE_FRAMES,
        "restart_every": 2 * (UNIQUE_FRAMES - 1),
        "l2": f"TSDF pair of {g.nvox * 8 / 1e6:.0f} MB (FP32) / {g.nvox * 4 / 1e6:.0f} MB (FP16) > 129 MB L2 "
              "(inputs larger than L2, no flush)",
        "parallelism": f"replicas x{args.gpus}",
    }


def cpu_baseline(cfg, frames, order, budget_s: float) -> dict:
    """The reference's kernel bodies compiled for this host's CPU (or the oracle port),
    frames/s over a bounded sample of the same sequence."""
    from oracle.pyoracle import GridSpec, Oracle, Reference

    g = cfg.grid
    gs = GridSpec(tuple(g.dims), tuple(g.start), g.voxel_size)
    ref = Reference.load()
    impl, kind = (ref, "reference") if ref is not None else (Oracle(), "port")
    H, W = cfg.camera.height, cfg.camera.width
    fresh = restarts(len(frames), len(order))
    pipe = impl.pipeline(H, W, gs, cfg.camera.K_reference())
    pipe.initial(frames[order[0]])
    n, t0 = 0, time.perf_counter()
    while n < len(order) - 1:
        k = 1 + n
        if fresh[k]:
            pipe.close()
            pipe = impl.pipeline(H, W, gs, cfg.camera.K_reference())
            pipe.initial(frames[order[k]])
        else:
            pipe.incoming(frames[order[k]])
        n += 1
        if time.perf_counter() - t0 >= budget_s and n >= 2:
            break
    dt = time.perf_counter() - t0
    cores = Oracle().lib.kfo_num_threads()
    pipe.close()
    return {"value": n / dt, "unit": "frames/s", "cores": cores, "kind": kind,
            "sample": f"{n} frames of {cfg.name} after the first (restarting every period like the GPU arm), {dt:.1f} s"}


def run_reference(args, dist: Dist):
    cfg = workload(args)
    if dist.rank != 0:
        dist.close()
        return
    from kinect_fusion_slam_gb300 import scene

    n_frames = min(args.steps + args.warmup + 1, UNIQUE_FRAMES)
    seq = scene.sequence(cfg, frames=n_frames)
    frames = seq.depths(n_frames)
    order = pingpong(n_frames, args.steps + args.warmup + 1)
    budget = max(10.0, min(120.0, args.cpu_seconds * 4))
    cb = cpu_baseline(cfg, frames, order, budget)
    line = {
        "metric": METRIC, "value": cb["value"], "unit": "frames/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 / cb["value"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded analytic room, Kinect v1 noise",
        "config": config_desc(cfg, args), "impl": "reference",
        "cpu_baseline": {k: cb[k] for k in ("kind", "cores", "sample")} | {"value": cb["value"], "unit": "frames/s"},
        "e2e": {"value": cb["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    dist.close()


def read_profile_traffic(stage_key: str):
    """DRAM bytes per frame of a stage from the committed ncu summary, if present."""
    p = ROOT / "profiles" / "ncu_traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == stage_key:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


FORMS = {
    # bit-exact drop-in: FP32 TSDF, the reference's 64-wide + serial summation order and
    # float Cholesky
    "plain": {"tsdf": "f32", "reduction": "reference", "solve": "reference"},
    # precision form: FP16 value + weight, compensated FP32 sums in one pass, FP64 solve
    "precision": {"tsdf": "f16", "reduction": "tree", "solve": "precise"},
}


def form_config(kf, cfg, form: str, **extra):
    g, cam = cfg.grid, cfg.camera
    f = FORMS[form]
    return kf.make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=g.start,
                          voxel_size=g.voxel_size,
                          tsdf_storage=kf.KF_TSDF_F16 if f["tsdf"] == "f16" else kf.KF_TSDF_F32,
                          icp_reduction=kf.KF_REDUCE_TREE if f["reduction"] == "tree" else kf.KF_REDUCE_REFERENCE_ORDER,
                          solve_mode=kf.KF_SOLVE_PRECISE if f["solve"] == "precise" else kf.KF_SOLVE_REFERENCE, **extra)


def trajectory_error(h, dev, fbytes, n_frames: int, workload_name: str = "c1"):
    """Absolute trajectory error (RMS and max translation difference, mm) of this handle's
    pipeline over frames 0..n-1 against the FP64 oracle's trajectory stored in
    tests/golden/fp64_<workload>_traj.npz; also the float oracle's (the reference's own
    arithmetic) error against the same trajectory."""
    p = ROOT / "tests" / "golden" / f"fp64_{workload_name}_traj.npz"
    if not p.exists():
        return None
    z = np.load(p)
    n = min(n_frames, int(z["frames"]))
    h.reset()
    poses = np.zeros((n, 4, 4))
    for k in range(n):
        ptr = dev.data_ptr() + k * fbytes
        (h.initial_processing_device if k == 0 else h.incoming_frame_device)(ptr)
        poses[k] = h.pose()
    p64 = z["poses64"][:n]
    p32 = z["poses32"][:n].astype(np.float64)
    e = np.linalg.norm(poses[:, :3, 3] - p64[:, :3, 3], axis=1)
    r = np.linalg.norm(p32[:, :3, 3] - p64[:, :3, 3], axis=1)

    def rpe(P):
        # relative pose error: RMS over frames of the translation difference between the
        # frame-to-frame motions inv(T[k-1]) T[k] of P and of the FP64 trajectory
        d = [np.linalg.inv(P[k - 1]) @ P[k] - np.linalg.inv(p64[k - 1]) @ p64[k] for k in range(1, n)]
        return float(np.sqrt(np.mean([np.sum(x[:3, 3] ** 2) for x in d])))

    return {"frames": n, "ate_mm": float(np.sqrt(np.mean(e ** 2))), "max_mm": float(e.max()), "rpe_mm": rpe(poses),
            "reference_float_ate_mm": float(np.sqrt(np.mean(r ** 2))), "reference_float_rpe_mm": rpe(p32)}


def synced_error(h, dev, fbytes, workload_name: str = "c1"):
    """Frame-synced accuracy against the FP64 oracle: for each frame k stored in
    tests/golden/fp64_<workload>_sync.npz the handle starts from the FP64 oracle's pose
    and surface prediction after frame k-1, runs frame k, and its pose is compared with
    the FP64 oracle's pose after frame k (translation mm, rotation mrad).  The same
    measure as tests/test_precision_synced.py (which runs the FP64 oracle live over 48
    frames); the float oracle's error from the same states is reported beside it."""
    p = ROOT / "tests" / "golden" / f"fp64_{workload_name}_sync.npz"
    if not p.exists():
        return None
    z = np.load(p)
    err = []
    for k, Tp, P, T64 in zip(z["frames"], z["poses_prev"], z["pred_prev"], z["poses"]):
        h.set_pose(Tp.astype(np.float32))
        h.set_predicted(P)
        h.incoming_frame_device(dev.data_ptr() + int(k) * fbytes)
        T = h.pose().astype(np.float64)
        R = T[:3, :3] @ T64[:3, :3].T
        sk = 0.5 * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
        err.append((float(np.linalg.norm(T[:3, 3] - T64[:3, 3])),
                    float(np.arctan2(np.linalg.norm(sk), (np.trace(R) - 1.0) / 2.0) * 1000.0)))
    e, fe = np.array(err), np.asarray(z["float_err"])
    return {"frames": [int(k) for k in z["frames"]], "max_mm": float(e[:, 0].max()),
            "rms_mm": float(np.sqrt(np.mean(e[:, 0] ** 2))), "max_mrad": float(e[:, 1].max()),
            "bar_mm": 1.0, "reference_float_max_mm": float(fe[:, 0].max()),
            "how": "each frame starts from the FP64 oracle's pose and prediction; pose after the frame vs the "
                   "FP64 oracle's (tests/test_precision_synced.py: all 48 c1 frames and 12 c2 frames, live oracle)"}


def run_form(args, dist, form, cfg, frames, order, fresh, stream, **extra):
    import torch

    import kinect_fusion_slam_gb300 as kf

    cam = cfg.camera
    h = kf.Handle(form_config(kf, cfg, form, **extra))
    K = cfg.camera.K_reference()
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    h.set_stream(stream.cuda_stream)
    dev = torch.from_numpy(frames.view(np.int16)).cuda()
    fbytes = cam.height * cam.width * 2
    n_total = 1 + args.warmup + args.steps

    def dptr(k):
        return dev.data_ptr() + order[k] * fbytes

    def device_step(k):
        if fresh[k]:
            if k:
                h.reset()
            h.initial_processing_device(dptr(k))
        else:
            h.incoming_frame_device(dptr(k))

    for k in range(0, 1 + args.warmup):
        device_step(k)
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(1 + args.warmup, n_total):
        device_step(k)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(e0.elapsed_time(e1))
    kpf = h.kernels_per_frame()
    n_fresh = sum(fresh[1 + args.warmup:n_total])
    # a restart: reset (two NaN fills or one for the FP16 pair, the state reset) and
    # InitialProcessing (vertex map, integration prep, box marks, mark list, integration,
    # ray cast)
    reset_kernels = 2 if FORMS[form]["tsdf"] == "f16" else 3
    launches = kpf * (args.steps - n_fresh) + (6 + reset_kernels) * n_fresh

    # per-stage device time with CUDA events recorded inside each frame's graph
    # (incoming frames only: InitialProcessing has no ICP stage)
    h.enable_stage_timing(True)
    stages = []
    for k in range(n_total, n_total + args.profile_frames):
        device_step(k)
        if not fresh[k]:
            stages.append(h.stage_times())
    h.enable_stage_timing(False)
    st = np.mean(np.array(stages), axis=0) if stages else np.zeros(5)
    stage_ms = {"vertex": float(st[0]), "icp": float(st[1]), "integration": float(st[2]), "raycast": float(st[3]),
                "frame": float(st[4])}

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        host = torch.from_numpy(frames.view(np.int16)).pin_memory()
        base = n_total + args.profile_frames
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(base, base + args.steps):
            ptr = host.data_ptr() + order[k] * fbytes
            if fresh[k]:
                h.reset()
                h.initial_processing_ptr(ptr)
            else:
                h.incoming_frame_ptr(ptr)
            h.pose()
        h.synchronize()  # the last frame's integration and ray cast (the pose is read at its ICP's end)
        dt = dist.max(time.perf_counter() - t0)
        e2e = {"value": args.steps * dist.world / dt, "unit": "frames/s", "h2d_bytes_per_step": fbytes,
               "d2h_bytes_per_step": 64}

    # integration's live voxels: those whose weight one incoming frame changes, counted
    # from the volume read back before and after it (outside every timed region)
    k = n_total + args.profile_frames + (0 if args.no_e2e else args.steps)
    while k < len(order) and fresh[k]:
        k += 1
    live = None
    if k < len(order) and getattr(args, "live_count", True):
        h.synchronize()
        _, w0 = h.volume()
        h.incoming_frame_device(dptr(k))
        h.synchronize()
        _, w1 = h.volume()
        live = int(np.count_nonzero(np.nan_to_num(w1, nan=-1.0) != np.nan_to_num(w0, nan=-1.0)))
        del w0, w1

    ate = trajectory_error(h, dev, fbytes, len(frames), cfg.name) if not args.no_ate else None
    sync = synced_error(h, dev, fbytes, cfg.name) if not args.no_ate else None
    h.close()
    return {"value": args.steps * dist.world / (ms_max / 1000.0), "ms_per_step": ms_max / args.steps,
            "e2e": e2e, "stages_ms": stage_ms, "gpu_launches": launches, "clocks": clk, "ate": ate,
            "live_voxels": live,
            "synced_fp64": sync, "tsdf": FORMS[form]["tsdf"]}


def roofline_of(cfg, r, form: str):
    """Roofline of the form's dominant stage, per frame, from the live stage events.

    Algorithmic bytes per frame: integration 16 B/voxel (FP32 pair) or 8 B/voxel (FP16
    pair) over the whole grid (the dense streaming figure); ray cast ~45 voxel reads of
    4 B (2 B FP16) per valid ray; ICP 49 B per pixel-iteration over 10 iterations.
    traffic: DRAM bytes per frame of that stage from the committed ncu launch list
    (cold-cache; the ICP maps stay in L2 in the running loop)."""
    g, cam = cfg.grid, cfg.camera
    tsdf = FORMS[form]["tsdf"]
    st = r["stages_ms"]
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    alg = {
        "integration": (16 if tsdf == "f32" else 8) * g.nvox,
        "icp": 49 * cam.height * cam.width * 10,
        "raycast": 45 * (4 if tsdf == "f32" else 2) * int(0.83 * cam.height * cam.width),
    }
    kernels = {"integration": "integrate_prep_kernel + integrate_mark_kernel + integrate_list_kernel + integrate_kernel",
               "icp": "10 x (icp_group_kernel + icp_solve_kernel)" if form == "plain" else "10 x icp_precise_kernel",
               "raycast": "raycast_kernel"}
    keys = {"integration": f"integration_{tsdf}", "icp": f"icp_{form}", "raycast": f"raycast_{tsdf}"}
    # what limits each stage (ncu evidence in profiles/): none of them is HBM-bound
    limiter = {"integration": "instruction issue: every voxel of the boxes marked from the depth tiles' frusta projected and tested",
               "icp": "latency: a serial chain of 10 association / reduction / solve passes, L2-resident",
               "raycast": "instruction issue (ALU pipe), L2-resident gathers"}
    stages = {}
    for s in ("integration", "icp", "raycast"):
        ach = alg[s] / (st[s] / 1000.0) / 1e9 if st[s] > 0 else 0.0
        stages[s] = {"achieved": ach, "frac": ach / peak, "ms": st[s], "alg_bytes": alg[s],
                     "traffic": read_profile_traffic(keys[s]), "traffic_source": "committed ncu summary",
                     "limiter": limiter[s]}
    # integration culls ~98 % of the grid: its dense 16 / 8 B per voxel is an equivalent
    # rate, not bytes moved; its DRAM traffic is the measured bytes
    ig = stages["integration"]
    ig["dense_equivalent_gbs"] = ig.pop("achieved")
    ig["dense_equivalent_frac"] = ig.pop("frac")
    ig["achieved"] = (ig["traffic"] / (st["integration"] / 1000.0) / 1e9
                      if ig["traffic"] and st["integration"] > 0 else None)
    ig["frac"] = ig["achieved"] / peak if ig["achieved"] else None
    # and the bytes of the voxels it actually updates (read and written, value + weight),
    # counted at run time
    if r.get("live_voxels"):
        ig["live_voxels"] = r["live_voxels"]
        ig["live_bytes"] = r["live_voxels"] * (16 if tsdf == "f32" else 8)
        ig["live_gbs"] = ig["live_bytes"] / (st["integration"] / 1000.0) / 1e9 if st["integration"] > 0 else None
        ig["live_frac"] = ig["live_gbs"] / peak if ig["live_gbs"] else None
    dom = max(stages, key=lambda s: stages[s]["ms"])
    return {"bound": "hbm", "achieved": stages[dom]["achieved"], "peak": peak, "unit": "GB/s",
            "frac": stages[dom]["frac"], "traffic": stages[dom]["traffic"], "kernel": kernels[dom],
            "limiter": stages[dom]["limiter"], "traffic_source": "committed ncu summary (profiles/ncu_traffic.txt)",
            "stage": dom, "per": "frame", "peak_source": "measured" if peaks else "fallback",
            "stages": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                       for k, v in stages.items()}}


def run_batching(args, stream) -> dict:
    """The batching form on c4: 16 scenes of uneven grids (128^3 @ 20 mm, 256^3 @ 15 mm,
    384x384x320 @ 10 mm) and depth sizes (640x480, 320x240), each its own seeded
    100-frame sequence (rendered in parallel on the host before the GPU work).  Every
    stage is one launch over all scenes, one graph per batch frame; integration and the
    ICP group pass run in either form (kf_batch_set_forms: one row of blocks per scene,
    or one fixed grid over all scenes' work) and both are timed, the faster kept.  Each
    batch frame is timed on the host from the call to its completion (the batch waits for
    the previous frame's table upload at every call, so frames do not overlap): that is
    every scene's latency in the batch.  Beside it the same scenes run one after another
    on their own handles, each frame timed the same way."""
    import torch

    import kinect_fusion_slam_gb300 as kf
    from kinect_fusion_slam_gb300 import scene

    cfgs = scene.batch_configs(16)
    nf = args.batch_frames
    depths = [torch.from_numpy(d.view(np.int16)).cuda() for d in scene.render_sequences(cfgs, nf)]
    confs = [kf.make_config(height=c.camera.height, width=c.camera.width, dims=c.grid.dims, grid_start=c.grid.start,
                            voxel_size=c.grid.voxel_size) for c in cfgs]
    fbytes = [c.camera.height * c.camera.width * 2 for c in cfgs]
    Ks = [c.camera.K_reference() for c in cfgs]

    def ptrs(k):
        return [d.data_ptr() + k * n for d, n in zip(depths, fbytes)]

    def pct(x):
        x = np.asarray(x) * 1000.0
        return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)), "mean": float(x.mean())}

    b = kf.Batch(confs)
    for h, K in zip(b.scenes, Ks):
        h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    forms = {"rows_per_scene": (False, False), "fixed_grid": (True, True)}
    res, tuning = {}, None
    for name, (pi, pc) in forms.items():
        for h in b.scenes:
            h.reset()
        b.set_forms(pi, pc)
        b.initial_processing_device(ptrs(0))
        b.synchronize()
        if tuning is None:
            tuning = b.autotune()
        lat = []
        t_all = time.perf_counter()
        for k in range(1, nf):
            t0 = time.perf_counter()
            b.incoming_frame_device(ptrs(k))
            b.synchronize()
            lat.append(time.perf_counter() - t0)
        t_all = time.perf_counter() - t_all
        res[name] = {"scene_frames_per_s": len(cfgs) * (nf - 1) / t_all, "batch_frame_latency_ms": pct(lat)}
    chosen = max(res, key=lambda k: res[k]["scene_frames_per_s"])
    kpf = b.kernels_per_frame()
    b.close()

    singles = [kf.Handle(c) for c in confs]
    for h, K in zip(singles, Ks):
        h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
        h.set_stream(stream.cuda_stream)
    for h, p in zip(singles, ptrs(0)):
        h.initial_processing_device(p)
    torch.cuda.synchronize()
    alone = [[] for _ in cfgs]
    t_all = time.perf_counter()
    for k in range(1, nf):
        for i, (h, p) in enumerate(zip(singles, ptrs(k))):
            t0 = time.perf_counter()
            h.incoming_frame_device(p)
            h.synchronize()
            alone[i].append(time.perf_counter() - t0)
    t_single = time.perf_counter() - t_all
    for h in singles:
        h.close()
    blat = res[chosen]["batch_frame_latency_ms"]
    per_scene = [{"scene": i, "grid": list(c.grid.dims), "voxel_mm": c.grid.voxel_size,
                  "image": [c.camera.width, c.camera.height], "batched_ms": {"p50": blat["p50"], "p99": blat["p99"]},
                  "alone_ms": {k: v for k, v in pct(alone[i]).items() if k != "mean"}} for i, c in enumerate(cfgs)]
    n = len(cfgs)
    return {"workload": "c4: 16 scenes, grids 128^3 @ 20 mm / 256^3 @ 15 mm / 384x384x320 @ 10 mm, "
                        "640x480 and 320x240 depth, single-level ICP x10, each scene its own 100-frame sequence",
            "scenes": n, "frames_per_scene": nf, "forms": res, "chosen_form": chosen,
            "scene_frames_per_s": res[chosen]["scene_frames_per_s"],
            "scene_frames_per_s_one_by_one": n * (nf - 1) / t_single,
            "speedup": res[chosen]["scene_frames_per_s"] / (n * (nf - 1) / t_single),
            "per_scene_latency_ms": per_scene, "kernels_per_batch_frame": kpf,
            "tuning": {"icp_group_warps": tuning[0], "ray_tile": ["8x4", "16x2", "4x8"][tuning[1]],
                       "ray_blocks_per_sm": tuning[2], "integration_z_chunk": tuning[3]}}


def run_differentiation(args) -> dict:
    """The differentiation form on c3: the seeded room's 64 frames fused by the library's
    integration into a 256^3 TSDF at 10 mm (diff.RoomWorkload), 64 perturbed starts (2-5
    cm, 1-3 degrees), 640x480 depth rendered and compared with the target rendered at the
    true pose under a Huber loss (delta 10 mm).  Device time per render and per adjoint
    (pose and voxel gradients; CUDA events), the pose gradient against central differences
    (step 1e-4 rad / 0.1 mm) at two starts, and 50 Huber Gauss-Newton steps from every
    start beside the reference's ICP from the same starts."""
    import torch

    from kinect_fusion_slam_gb300 import diff

    delta = 10.0
    w = diff.RoomWorkload("c3")
    targets = [diff.render(w.desc, w.tsdf, T)[0].double() for T in w.poses]
    grads = []
    for T, tg in zip(w.starts, targets):
        depth, _ = diff.render(w.desc, w.tsdf, T)
        _, psi = diff.huber(depth.double() - tg, delta)
        grads.append((psi * (tg > 0)).float())
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    for T, gD in zip(w.starts[:3], grads):
        diff.render(w.desc, w.tsdf, T)
        diff.render_backward(w.desc, w.tsdf, T, gD, None)
    torch.cuda.synchronize()
    e[0].record()
    for T in w.starts:
        diff.render(w.desc, w.tsdf, T)
    e[1].record()
    for T, gD in zip(w.starts, grads):
        diff.render_backward(w.desc, w.tsdf, T, gD, None)
    e[2].record()
    torch.cuda.synchronize()
    n = len(w.starts)

    # the pose gradient against central differences, on pixels whose crossing stays
    # between the same two samples of the march in every evaluation
    def bracket(depth):
        return torch.floor((depth.double() - w.desc.t_near) / w.desc.step)

    def stable(depth, b0):
        b = bracket(depth)
        f = (depth.double() - w.desc.t_near) / w.desc.step - b
        return (depth > 0) & (f > 0.05) & (f < 0.95) & (b == b0)

    eps = np.array([1e-4] * 3 + [0.1] * 3)
    rel = []
    for k in (0, 32):
        T, tg = w.starts[k], targets[k]
        poses = [T] + [diff.se3_exp(sg * eps[q] * np.eye(6)[q]) @ T for q in range(6) for sg in (1, -1)]
        mask = tg > 0
        b0 = bracket(diff.render(w.desc, w.tsdf, T)[0])
        for P in poses:
            mask &= stable(diff.render(w.desc, w.tsdf, P)[0], b0)
        mask = mask.double()

        def loss(P):
            return float((diff.huber(diff.render(w.desc, w.tsdf, P)[0].double() - tg, delta)[0] * mask).sum())

        _, psi = diff.huber(diff.render(w.desc, w.tsdf, T)[0].double() - tg, delta)
        _, g6 = diff.render_backward(w.desc, w.tsdf, T, (psi * mask).float(), None, want_tsdf=False)
        fd = np.array([(loss(poses[1 + 2 * q]) - loss(poses[2 + 2 * q])) / (2 * eps[q]) for q in range(6)])
        rel.append(float(np.max(np.abs(g6.double().cpu().numpy() - fd)) / np.abs(fd).max()))

    # the depth Jacobian against the point-to-plane ICP row -[x cross m, m]/(m.r) on
    # locally flat pixels (rendered normal within 3 degrees over 9x9) at the first pose
    T = w.poses[0]
    depth, normal = diff.render(w.desc, w.tsdf, T)
    nrm, dep = normal.double().cpu().numpy(), depth.cpu().numpy()
    Ki = np.linalg.inv(np.asarray(w.K, np.float64))
    p2p = []
    for v in range(40, dep.shape[0] - 40, 11):
        for u in range(40, dep.shape[1] - 40, 14):
            if dep[v, u] <= 0 or not np.all(dep[v - 4:v + 5, u - 4:u + 5] > 0):
                continue
            m = nrm[v, u] / np.linalg.norm(nrm[v, u])
            if (nrm[v - 4:v + 5, u - 4:u + 5] @ m).min() < np.cos(np.radians(3.0)):
                continue
            g1 = torch.zeros_like(depth)
            g1[v, u] = 1.0
            _, gp = diff.render_backward(w.desc, w.tsdf, T, g1, None, want_tsdf=False)
            r = T[:3, :3] @ (Ki @ np.array([u + 1.0, v + 1.0, 1.0]))
            x = T[:3, 3] + float(dep[v, u]) * r
            want = -np.concatenate([np.cross(x, m), m]) / float(m @ r)
            p2p.append(float(np.linalg.norm(gp.double().cpu().numpy() - want) / np.linalg.norm(want)))

    steps = 50
    ref, icp = [], []
    t0 = time.perf_counter()
    for k, T0 in enumerate(w.starts):
        T, _ = diff.refine_pose(w.desc, w.tsdf, T0, targets[k].float(), iterations=steps, max_residual=0.0,
                                huber_delta=delta)
        ref.append(diff.pose_error(T, w.poses[k]))
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    for k, T0 in enumerate(w.starts):
        icp.append(diff.pose_error(diff.icp_align(w.handle, T0, targets[k].cpu().numpy()), w.poses[k]))
    t_icp = time.perf_counter() - t0
    start_err = np.array([diff.pose_error(T0, T) for T0, T in zip(w.starts, w.poses)])
    observed = int(torch.isfinite(w.tsdf).sum())
    w.close()
    ref, icp = np.array(ref), np.array(icp)

    def summary(err):
        return {"success_rate": float(np.mean((err[:, 0] <= 2.0) & (err[:, 1] <= 0.2))),
                "median_mm": float(np.median(err[:, 0])), "median_deg": float(np.median(err[:, 1])),
                "max_mm": float(err[:, 0].max())}

    return {"workload": "c3: 256^3 TSDF @ 10 mm fused from 64 frames of the seeded room by the library's integration, "
                        "640x480 render, 64 poses perturbed 2-5 cm / 1-3 deg, Huber loss delta 10 mm",
            "observed_voxels": observed, "render_ms": e[0].elapsed_time(e[1]) / n,
            "adjoint_ms": e[1].elapsed_time(e[2]) / n,
            "pose_gradient_vs_central_differences": {"step": "1e-4 rad, 0.1 mm", "max_rel_error": max(rel)},
            "depth_jacobian_vs_point_to_plane_row": {"pixels": len(p2p), "median_rel_diff": float(np.median(p2p)),
                                                     "p90_rel_diff": float(np.percentile(p2p, 90))},
            "start_error_median_mm": float(np.median(start_err[:, 0])),
            "start_error_median_deg": float(np.median(start_err[:, 1])),
            "refinement": {"steps": steps, "ms_per_step": 1000.0 * t_ref / (n * steps), **summary(ref)},
            "icp": {"iterations": 10, "ms_per_alignment": 1000.0 * t_icp / n, **summary(icp)},
            "success": "final error <= 2 mm and <= 0.2 deg"}


def run_precision_c2(args, dist, stream) -> dict:
    """Both forms on c2, the precision form's own workload: 640x480 depth into the
    512x512x430 grid at 7 mm (113 M voxels: 902 MB as the FP32 pair, 451 MB as FP16),
    the same seeded room, noise and frame order as c1; frames/s with the depth frames in
    device memory, and the trajectory error of the first 48 frames against the FP64
    oracle's (tests/golden/fp64_c2_traj.npz)."""
    from kinect_fusion_slam_gb300 import scene

    cfg = scene.config("c2")
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.profile_frames, sub.no_e2e, sub.live_count = 100, 3, 5, True, False
    n_all = 1 + sub.warmup + sub.steps + sub.profile_frames + 4
    seq = scene.sequence(cfg, frames=UNIQUE_FRAMES)
    frames = seq.depths(UNIQUE_FRAMES)
    order = pingpong(UNIQUE_FRAMES, n_all)
    fresh = restarts(UNIQUE_FRAMES, n_all)
    out = {"workload": "c2: 640x480 uint16 depth, 512x512x430 TSDF @ 7 mm, single-level ICP x10",
           "steps": sub.steps}
    for form in ("precision", "plain"):
        r = run_form(sub, dist, form, cfg, frames, order, fresh, stream)
        out[form] = {"frames_per_s": r["value"], "stages_ms": r["stages_ms"], "ate": r["ate"]}
    out["speedup_vs_fp32_form"] = out["precision"]["frames_per_s"] / out["plain"]["frames_per_s"]
    return out


def run_pyramid_c1(args, dist, stream) -> dict:
    """Both forms on c1 with the three-level ICP pyramid of the workload's description
    (10/5/4 iterations, coarsest level first).  The reference has one level (10
    iterations), which the headline line and its reference arm keep; this times the
    pyramid form beside it, with the depth frames in device memory."""
    from kinect_fusion_slam_gb300 import scene

    cfg = scene.config("c1")
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.profile_frames, sub.no_e2e, sub.no_ate, sub.live_count = 100, 3, 5, True, True, False
    n_all = 1 + sub.warmup + sub.steps + sub.profile_frames + 4
    seq = scene.sequence(cfg, frames=UNIQUE_FRAMES)
    frames = seq.depths(UNIQUE_FRAMES)
    order = pingpong(UNIQUE_FRAMES, n_all)
    fresh = restarts(UNIQUE_FRAMES, n_all)
    out = {"workload": "c1 with a 3-level ICP pyramid (10/5/4 iterations)", "steps": sub.steps}
    for form in ("precision", "plain"):
        r = run_form(sub, dist, form, cfg, frames, order, fresh, stream, icp_levels=3, icp_iterations=(10, 5, 4))
        out[form] = {"frames_per_s": r["value"], "stages_ms": r["stages_ms"]}
    return out


def run_gb300(args, dist: Dist):
    import torch

    from kinect_fusion_slam_gb300 import scene

    torch.cuda.set_device(dist.local_rank)
    cfg = workload(args)
    n_total = 1 + args.warmup + args.steps
    seq = scene.sequence(cfg, frames=UNIQUE_FRAMES)
    frames = seq.depths(UNIQUE_FRAMES)
    # and a few frames more for the live-voxel count (run_form)
    n_all = n_total + args.profile_frames + (0 if args.no_e2e else args.steps) + 4
    order = pingpong(UNIQUE_FRAMES, n_all)
    fresh = restarts(UNIQUE_FRAMES, n_all)
    # a dedicated stream: torch's default stream is the legacy NULL stream (handle 0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    forms = ["precision", "plain"] if args.form == "both" else [args.form]
    res = {f: run_form(args, dist, f, cfg, frames, order, fresh, stream) for f in forms}
    head = res[forms[0]]

    extra = {}
    if not args.no_extra_forms and dist.world == 1:
        extra["batching_c4"] = run_batching(args, stream)
        extra["differentiation_c3"] = run_differentiation(args)
        extra["precision_c2"] = run_precision_c2(args, dist, stream)
        extra["pyramid_c1"] = run_pyramid_c1(args, dist, stream)

    cb = None
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(cfg, frames, order, args.cpu_seconds)

    # config names the workload only (the same dict as the reference arm's line); the form
    # that produced `value` is a key of its own
    desc = config_desc(cfg, args)
    line = {
        "metric": METRIC, "value": head["value"], "unit": "frames/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 arithmetic, " + ("f16 TSDF value+weight" if head["tsdf"] == "f16" else "f32 TSDF"),
        "data": "synthetic: seeded analytic room, Kinect v1 noise", "config": desc,
        "form": forms[0], "tsdf_storage": head["tsdf"],
        "roofline": roofline_of(cfg, head, forms[0]), "cpu_baseline": cb, "e2e": head["e2e"],
        "gpu_launches": head["gpu_launches"], "clocks": head["clocks"], "stages_ms": head["stages_ms"],
        "ate": head["ate"], "synced_fp64": head["synced_fp64"],
    }
    if "plain" in res and forms[0] != "plain":
        p = res["plain"]
        line["fp32_form"] = {"value": p["value"], "ms_per_step": p["ms_per_step"], "e2e": p["e2e"],
                             "stages_ms": p["stages_ms"], "ate": p["ate"], "synced_fp64": p["synced_fp64"],
                             "gpu_launches": p["gpu_launches"],
                             "roofline": roofline_of(cfg, p, "plain")}
        line["speedup_vs_fp32_form"] = head["value"] / p["value"]
        line["gpu_launches"] = head["gpu_launches"] + p["gpu_launches"]
    line.update(extra)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def main(argv=None):
    args = parse_args(argv)
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_gb300(args, dist)


if __name__ == "__main__":
    main()
