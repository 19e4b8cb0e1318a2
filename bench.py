"""Benchmark of the fine-stage training iteration (and the merged-VDB render).

Workload (one "step"): one fine-stage iteration of PlenVDB's DVGO training on
8192 rays over a 160^3 sparse scene (8 seeded ellipsoids, ~10% voxels active,
8^3 leaves), k0 = 12 channels, rgbnet 39-128-128-3, per-voxel Adam on both
grids (skip-zero-grad), Adam on the rgbnet, TV weight 1e-4, in FP32 (the plain
method) or BF16 (--precision bf16). Synthetic seeded data stands in for the
NeRF datasets; targets are rendered from a seeded ground-truth grid.

Beside the headline line's step timing the JSON carries: per-stage times and
rooflines, the end-to-end number through the public API with host buffers,
the merged-VDB render of 200 800x800 frames (FP32 plain and BF16), the PSNR
of FP32- and BF16-trained models after 2000 iterations on 8 held-out 800x800
views, the 320^3 / 65536-ray BF16 training step, and `lifecycle`: the steps
around the training step (merged compression, 80^3 -> 160^3 rescaling, the
mask-cache update, rays of a view, the in-mask-cache hit test, ray
compaction, per-view voxel counts) with device time, algorithmic bytes,
fraction of the measured HBM bandwidth and the oracle's CPU time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --lifecycle-only      # just the lifecycle timings

Prints one JSON line (rank 0). Under torchrun every rank runs an independent
replica (the path has no cross-GPU exchange in this build) and the time is the
max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RAYS = 8192
RESO = 160
N_BATCHES = 8
METRIC = "fine-stage train it/s @8192 rays (160^3, k0=12, rgbnet 39-128-128-3)"
WORKLOAD = (f"fine-stage iteration, {RAYS} rays, {RESO}^3 sparse VDB (8^3 leaves, 8 seeded "
            "ellipsoids), k0=12, rgbnet 39-128-128-3, TV 1e-4")
L2_NOTE = ("GPU: a 512 MB buffer (> 129 MB L2) is written between timed steps, outside the "
           "step events")


def workload_config(active_fraction):
    """The workload both arms time (the same dict in both JSON lines)."""
    return {"workload": WORKLOAD, "rays": RAYS, "reso": RESO,
            "scene": "union of 8 seeded ellipsoids (centres U[-1,1]^3, radii U[0.15,0.5], "
                     "scene seed 0), raw density N(2,1), k0 N(0,0.1), background -10",
            "active_fraction": round(float(active_fraction), 4),
            "batches": f"{N_BATCHES} seeded batches of {RAYS} rays over 100 views (ray seed 1), "
                       "taken in turn",
            "targets": "rendered from a seeded ground-truth model (value seed 4242, rgbnet "
                       "seed 99) through the same forward",
            "density_only": f"{RAYS} rays, alpha = 1 - alphainv_last vs U[0,1] (seed 3), "
                            "forward + backward, no optimiser",
            "l2": L2_NOTE}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp32", "bf16"], default="bf16",
                    help="bf16: BF16 rgbnet on the tensor cores (the FP32 plain method is "
                         "timed beside it); fp32: the plain method alone")
    ap.add_argument("--render-frames", type=int, default=200)
    ap.add_argument("--psnr-iters", type=int, default=2000,
                    help="training iterations of the BF16-vs-FP32 PSNR run (0: skip)")
    ap.add_argument("--no-fp32-plain", action="store_true",
                    help="skip the FP32 plain-method leg of a --precision bf16 run")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the 320^3 / 65536-ray training measurement")
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--no-lifecycle", action="store_true",
                    help="skip the timings of the steps around the training step")
    ap.add_argument("--lifecycle-only", action="store_true",
                    help="only the lifecycle timings (for profiling their kernels)")
    ap.add_argument("--large-only", action="store_true",
                    help="only the 320^3 / 65536-ray training measurement (for profiling "
                         "its kernels)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the fused step eagerly instead of replaying a CUDA graph")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_throughput(step_ms_total, steps, world, device="cuda"):
    """Whole-job it/s of `world` independent replicas (the path has no
    cross-GPU exchange): every replica runs `steps` steps, the job's time is
    the slowest replica's (max over ranks), value = world * steps / time.
    Returns (value, ms_per_step of the slowest replica)."""
    import torch
    import torch.distributed as dist
    t = float(step_ms_total)
    if world > 1:
        x = torch.tensor([t], device=device, dtype=torch.float64)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return world * steps / (t / 1e3), t / steps


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region.

    nvidia-smi starts before the warm-up steps and polls every 200 ms with its
    output line-buffered (stdbuf, where present); every sample carries
    nvidia-smi's timestamp. begin() and end() mark the timed region on the
    same clock, and the summary keeps the samples taken inside it plus the
    first one after it (which covers the region's tail), so a region shorter
    than one interval still gets the sample that spans it."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 200

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        import shutil
        cmd = ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
               "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)]
        if shutil.which("stdbuf"):
            cmd = ["stdbuf", "-oL"] + cmd
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_ready(self, timeout: float = 10.0):
        """Until nvidia-smi has printed its first sample (it takes a moment to start)."""
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.01)

    def begin(self):
        import datetime
        self.t0 = datetime.datetime.now()

    def end(self):
        import datetime
        self.t1 = datetime.datetime.now()

    @staticmethod
    def _stamp(text):
        import datetime
        try:
            return datetime.datetime.strptime(text.strip(), "%Y/%m/%d %H:%M:%S.%f")
        except ValueError:
            return None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # wait for the first sample after the region (it covers the region's tail)
        t_wait = time.time()
        while time.time() - t_wait < 2.0:
            last = self._stamp(self.lines[-1].split(",")[0]) if self.lines else None
            if last is not None and self.t1 is not None and last > self.t1:
                break
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            ts = self._stamp(parts[0])
            if ts is None:
                continue
            rows.append((ts, parts))
        inside = [r for r in rows if self.t0 <= r[0] <= self.t1]
        after = [r for r in rows if r[0] > self.t1]
        picked = inside + after[:1]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, parts in picked:
            try:
                sm.append(float(parts[2]))
                smax.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "samples_inside": len(inside), "interval_ms": self.INTERVAL_MS}


class NvmlSampler:
    """SM clock and clock-event reasons read through NVML (ctypes on the
    driver's libnvidia-ml, read-only queries) every millisecond from a thread
    while the timed region runs: a region of a few tens of milliseconds gets
    tens of samples, where nvidia-smi's interval gets none."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        import ctypes
        self.ok = False
        self.samples = []
        try:
            self.nv = ctypes.CDLL("libnvidia-ml.so.1")
            if self.nv.nvmlInit_v2() != 0:
                return
            self.h = ctypes.c_void_p()
            if self.nv.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(self.h)) != 0:
                return
            self.reason_fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = ctypes.c_uint()
            self.max_mhz = (float(mx.value) if self.nv.nvmlDeviceGetMaxClockInfo(
                self.h, 1, ctypes.byref(mx)) == 0 else None)
            self.ok = True
        except Exception:
            self.ok = False

    def _run(self):
        import ctypes
        mhz, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.halt:
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(mhz)) == 0 and \
                    self.reason_fn(self.h, ctypes.byref(rs)) == 0:
                self.samples.append((float(mhz.value), int(rs.value)))
            time.sleep(0.001)

    def begin(self):
        if not self.ok:
            return
        self.halt = False
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def end(self):
        if not self.ok:
            return {"samples": 0, "note": "NVML unavailable"}
        self.halt = True
        self.thread.join(timeout=1.0)
        mask = 0
        for _, r in self.samples:
            mask |= r
        return {"samples": len(self.samples),
                "sm_mhz": float(np.median([m for m, _ in self.samples])) if self.samples else None,
                "sm_mhz_min": min((m for m, _ in self.samples), default=None),
                "sm_max_mhz": self.max_mhz,
                "reasons": sorted(n for b, n in self.REASONS.items() if mask & b)}


# ------------------------------------------------------------------ setup
def make_problem(device_seed=0):
    import torch

    from plenvdb_gb300.march import CompositeFn, MarchSample, MarchWorkspace, RgbNetFn, march_params
    from plenvdb_gb300.scene import (CameraConfig, SceneConfig, build_grids, random_rays,
                                     rgbnet_init)
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=RESO, n_ellipsoids=8, seed=0)
    cfg = FineStageConfig(reso=RESO)
    cam = CameraConfig()
    n_batches = N_BATCHES
    ro, rd, vd = random_rays(cam, RAYS * n_batches, 100, seed=1 + device_seed)
    # ground-truth targets: a second seeded grid + rgbnet rendered by the same march
    gd, gk = build_grids(scfg, value_seed=4242)
    gt_net = [p.cuda() for p in rgbnet_init(seed=99)]
    ws = MarchWorkspace(RAYS, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
    p = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                     cfg.interval, cfg.fast_color_thres, cfg.bg)
    targets = []
    dummy = torch.zeros(1, device="cuda")
    with torch.no_grad():
        for b in range(n_batches):
            sl = slice(b * RAYS, (b + 1) * RAYS)
            tro, trd, tvd = (torch.from_numpy(a[sl]).cuda() for a in (ro, rd, vd))
            w, last, k0, _ = MarchSample.apply(dummy, ws, gd, gk, tro, trd, p)
            rgb = RgbNetFn.apply(k0, tvd, ws, 4, 0, *gt_net)
            targets.append(CompositeFn.apply(w, rgb, last, ws, cfg.bg).clone())
    del gd, gk, ws
    tgt = torch.cat(targets).cpu().numpy()
    return scfg, cfg, cam, ro, rd, vd, tgt


def flush_l2(buf):
    buf.add_(1.0)  # write 512 MB (> 129 MB L2) between timed steps


def run_ours(args):
    import torch
    import torch.distributed as dist

    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.scene import build_grids, rgbnet_init
    from plenvdb_gb300.trainer import FineStageTrainer

    ws_, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws_ > 1:
        dist.init_process_group("nccl", init_method="env://")
    lib = L.load()
    scfg, cfg, cam, ro, rd, vd, tgt = make_problem(device_seed=rank)
    cfg.precision = 1 if args.precision == "bf16" else 0
    cfg.use_graph = not args.no_graph
    dg, kg = build_grids(scfg)
    tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2), cfg, max_rays=RAYS)
    nb = ro.shape[0] // RAYS
    dev = [tuple(torch.from_numpy(a[b * RAYS:(b + 1) * RAYS]).cuda() for a in (ro, rd, vd, tgt))
           for b in range(nb)]
    flush = torch.zeros(128 * 1024 * 1024, device="cuda")
    st = torch.cuda.current_stream()
    clocks = ClockSampler(local)
    clocks.start()
    for i in range(args.warmup):
        tr.step(*dev[i % nb])
    torch.cuda.synchronize()
    clocks.wait_ready()
    # ---------------- timed region (device-resident inputs)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    launches0 = lib.pvdb_launch_count()
    if ws_ > 1:
        dist.barrier()
    nvml = NvmlSampler(local)
    torch.cuda.synchronize()
    clocks.begin()
    nvml.begin()
    t_wall = time.perf_counter()
    for i in range(args.steps):
        flush_l2(flush)
        evs[i][0].record(st)
        loss = tr.step(*dev[(args.warmup + i) % nb])
        evs[i][1].record(st)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    nv_clk = nvml.end()
    clocks.end()
    launches = lib.pvdb_launch_count() - launches0
    clk = clocks.stop()
    clk["nvml_inside"] = nv_clk
    if nv_clk.get("samples"):
        # the in-region samples are the record; nvidia-smi's stay beside them
        clk["sm_mhz"] = nv_clk["sm_mhz"]
        clk["sm_max_mhz"] = nv_clk["sm_max_mhz"] or clk["sm_max_mhz"]
        clk["reasons"] = sorted(set(clk["reasons"]) | set(nv_clk["reasons"]))
    step_ms = float(sum(a.elapsed_time(b) for a, b in evs))
    value, ms_per_step = replica_throughput(step_ms, args.steps, ws_)
    stage_ms = stage_profile(tr, dev, nb, flush, args)
    staging = leaf_staging_compare(tr, dev, nb, flush, args, stage_ms)
    # ---------------- the FP32 plain method on the same workload, same timing
    plain = None
    if args.precision == "bf16" and not args.no_fp32_plain:
        import dataclasses
        pcfg = dataclasses.replace(cfg, precision=0)
        pdg, pkg = build_grids(scfg)
        ptr = FineStageTrainer(pdg, pkg, rgbnet_init(seed=2), pcfg, max_rays=RAYS)
        for i in range(args.warmup):
            ptr.step(*dev[i % nb])
        psteps = min(args.steps, 30)
        pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(psteps)]
        torch.cuda.synchronize()
        for i in range(psteps):
            flush_l2(flush)
            pev[i][0].record(st)
            ptr.step(*dev[(args.warmup + i) % nb])
            pev[i][1].record(st)
        torch.cuda.synchronize()
        pms = float(sum(a.elapsed_time(b) for a, b in pev)) / psteps
        plain = {"it_s": 1e3 / pms, "ms_per_step": pms, "steps": psteps,
                 "speedup_bf16": value * pms / 1e3}
        del ptr, pdg, pkg
    # ---------------- the plain FP32 density-only forward + backward
    dens_only = run_density_only(scfg, cfg, dev, args, flush)
    # ---------------- end to end through the public API with host buffers
    e2e = run_e2e(tr, ro, rd, vd, tgt, args, flush)
    # ---------------- roofline of the dominant stage
    roof = roofline(stage_ms, tr, scfg)
    # ---------------- render FPS: 800x800 frames from the merged index
    render = None if args.no_render else run_render(scfg, cfg, cam, tr, args)
    # ---------------- BF16 vs FP32 quality after training from one seed
    psnr = run_psnr(scfg, cfg, cam, args.psnr_iters) if args.psnr_iters > 0 else None
    # ---------------- the steps around the training step (lifecycle)
    life = None if args.no_lifecycle else run_lifecycle(scfg, cfg, cam, tr)
    # ---------------- 320^3 grid, 65536 rays per step
    large = None if args.no_large else run_large(args)
    out = None
    if rank == 0:
        from plenvdb_gb300.scene import scene_mask
        af = float(scene_mask(scfg).mean())
        out = {
            "metric": METRIC, "value": value, "unit": "it/s", "n_gpus": ws_,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "bf16+f32",
            "precision": (args.precision if args.precision == "fp32" else
                          "bf16: BF16 k0 features and rgbnet, FP32 accumulation, density, "
                          "transmittance, Adam moments and master values"),
            "data": "synthetic: seeded 8-ellipsoid 160^3 scene, 100 seeded 800x800 views, "
                    "targets rendered from a seeded ground-truth grid",
            "config": workload_config(af),
            "parallelism": "replicas" if ws_ > 1 else "single GPU",
            "launch": "eager" if args.no_graph else "CUDA graph replay of the fused step",
            "wall_s": t_wall, "clocks": clk, "gpu_launches": int(launches),
        }
        # short scalars first (the headline's context), then the large objects
        if plain:
            out["fp32_plain_it_s"] = plain["it_s"]
            out["bf16_over_fp32"] = plain["speedup_bf16"]
        if psnr:
            out["psnr_delta_db"] = psnr["delta_db"]
        if render:
            out["render_fps_bf16"] = render["bf16"]["fps"]
            out["render_fps_fp32"] = render["fp32"]["fps"]
        out["density_only_it_s"] = dens_only["it_s"]
        out["density_only_rays_s"] = dens_only["rays_per_s"]
        out["roofline"] = roof
        out["e2e"] = e2e
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(scfg, cfg, cam, ro, rd, vd, tgt, tr, args)
        out["stage_ms"] = stage_ms
        out["leaf_staging"] = staging
        if plain:
            out["fp32_plain"] = plain
        out["density_only"] = dens_only
        if render:
            out["render"] = render
        if psnr:
            out["psnr"] = psnr
        if large:
            out["large"] = large
        if life:
            out["lifecycle"] = life
        print(json.dumps(out), flush=True)
    if ws_ > 1:
        dist.barrier()
        dist.destroy_process_group()


def stage_profile(tr, dev, nb, flush, args, n=None):
    """Per-stage device time from events between the stages of eagerly launched
    steps (a graph replay has no stage boundaries); a separate, shorter pass
    after the timed region."""
    import ctypes
    import torch
    from plenvdb_gb300 import _lib as L
    n = n or max(5, min(args.steps, 20))
    use_graph = tr.tc.use_graph
    tr.tc.use_graph = 0
    L.call("pvdb_profile_begin", n)
    for i in range(n):
        if flush is not None:
            flush_l2(flush)
        tr.step(*dev[i % nb])
    torch.cuda.synchronize()
    marks = (ctypes.c_float * 16)()
    ncalls = ctypes.c_int32()
    L.call("pvdb_profile_end", marks, 16, ctypes.byref(ncalls))
    tr.tc.use_graph = use_graph
    stage_names = {1: "march_fwd", 2: "k0_gather", 3: "rgbnet_fwd", 4: "composite_loss",
                   5: "rgbnet_bwd", 6: "march_bwd", 7: "cell_grouping", 8: "voxel_gather",
                   9: "tv", 10: "voxel_adam", 11: "rgbnet_adam"}
    return {stage_names[i]: marks[i] / max(1, ncalls.value) for i in stage_names}


def leaf_staging_compare(tr, dev, nb, flush, args, stage_ms, n=None):
    """The march forward stage with the density leaves staged in shared memory
    by bulk copies (pvdb_march_set_leaf_staging) against the default pass,
    from the same eager stage profile; staging is switched off again."""
    tr.ws.set_leaf_staging(True)
    try:
        sm = stage_profile(tr, dev, nb, flush, args, n=n)
    finally:
        tr.ws.set_leaf_staging(False)
    return {"march_fwd_ms_default": stage_ms["march_fwd"], "march_fwd_ms_staged": sm["march_fwd"],
            "note": "density leaves of each ray's evaluated samples copied into shared memory "
                    "with cp.async.bulk (24 slots of 2 KB per ray block); off by default"}


def run_e2e(tr, ro, rd, vd, tgt, args, flush):
    """Same iteration through FineStageTrainer.step with pinned host inputs copied
    H2D every step and the loss read back D2H every step."""
    import torch
    st = torch.cuda.current_stream()
    nb = ro.shape[0] // RAYS
    host = [tuple(torch.from_numpy(np.ascontiguousarray(a[b * RAYS:(b + 1) * RAYS])).pin_memory()
                  for a in (ro, rd, vd, tgt)) for b in range(nb)]
    dev = [torch.empty(RAYS, 3, device="cuda") for _ in range(4)]
    loss_h = torch.empty(1).pin_memory()
    steps = max(10, args.steps // 2)
    for i in range(3):
        for d, h in zip(dev, host[i % nb]):
            d.copy_(h, non_blocking=True)
        tr.step(*dev)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for i in range(steps):
        flush_l2(flush)
        evs[i][0].record(st)
        for d, h in zip(dev, host[i % nb]):
            d.copy_(h, non_blocking=True)
        loss = tr.step(*dev)
        loss_h.copy_(loss, non_blocking=True)
        evs[i][1].record(st)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    return {"value": 1e3 / ms, "unit": "it/s", "ms_per_step": ms,
            "h2d_bytes_per_step": int(sum(t.numel() * 4 for t in host[0])),
            "d2h_bytes_per_step": 4}


def run_density_only(scfg, cfg, dev, args, flush):
    """The plain FP32 density-only forward + backward (the configuration the
    reference's CPU path can also run): 8192 rays through the density march
    (no k0 grid), composited alpha = 1 - alphainv_last against a seeded U[0,1]
    target, loss mean((alpha - target)^2), and its backward into the density
    grid's gradient (zeroed each step). C-ABI calls on the current stream, no
    host synchronisation inside a step; CUDA events per step, L2 flushed
    between steps."""
    import ctypes
    import torch

    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import MarchWorkspace, march_params
    from plenvdb_gb300.plenvdb import device_view
    from plenvdb_gb300.scene import build_grids
    dg, _ = build_grids(scfg)
    ws = MarchWorkspace(RAYS, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
    p = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                     cfg.interval, cfg.fast_color_thres, cfg.bg, cfg.t_stop)
    tgt = torch.from_numpy(np.random.default_rng(3).random(RAYS).astype(np.float32)).cuda()
    v = ws.views()
    last = device_view(v.alphainv_last, (RAYS,), "float32", ws)
    g_last = torch.empty(RAYS, device="cuda")
    loss = torch.empty((), device="cuda")
    st = torch.cuda.current_stream()

    def step(b):
        ro, rd = dev[b][0], dev[b][1]
        L.call("pvdb_grid_zero_grad", dg.handle, L.stream_of())
        L.call("pvdb_march_forward", ws.h, dg.handle, None, L.ptr(ro), L.ptr(rd), RAYS,
               ctypes.byref(p), None, None, L.stream_of())
        err = (1.0 - last) - tgt
        torch.mean(err * err, out=loss)
        torch.mul(err, -2.0 / RAYS, out=g_last)
        L.call("pvdb_march_backward", ws.h, dg.handle, None, None, L.ptr(g_last), None,
               L.stream_of())

    nb = len(dev)
    for i in range(max(args.warmup, 3)):
        step(i % nb)
    torch.cuda.synchronize()
    steps = max(10, min(args.steps, 50))
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for i in range(steps):
        flush_l2(flush)
        evs[i][0].record(st)
        step(i % nb)
        evs[i][1].record(st)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    kept, rows, evaluated = ws.stats()
    return {"it_s": 1e3 / ms, "rays_per_s": RAYS * 1e3 / ms, "ms_per_step": ms, "steps": steps,
            "loss": float(loss.item()), "kept_samples": kept, "evaluated_samples": evaluated,
            "precision": "fp32",
            "timing": "CUDA events per step on the launching stream, L2 flushed between steps"}


# Algorithmic work per unit of each train-step stage:
#   march_fwd       36 B per evaluated sample (8 density corners + the alpha)
#   k0_gather       8*C*e + 16 B per colour row (8 k0 corners of e-byte
#                   features + row record)
#   rgbnet_fwd      36,608 FLOP per row + 6,912 per ray (PE part of layer 0)
#   rgbnet_bwd      73,216 FLOP per row: twice the forward's 36,608 (the
#                   activation and weight gradients); the layer-0/1 recompute
#                   and the MMA padding are executed work, reported apart
#   march_bwd       120 B per kept sample (saved alpha/weight/step/row, grad,
#                   8 density corners, 64 B gradient record, 4 B key)
#   cell_grouping   32 B per kept sample (key read twice, rank written and read,
#                   cell offset read, grouped key and index written)
#   voxel_gather    64 B record + 8 corner gradients (1 + C floats) per kept sample
#   tv              8 B per visited voxel-channel: the sparse TV terms (value
#                   read, term written; the six neighbour reads are cache hits);
#                   visited = the active voxels of the touched leaves
#   voxel_adam      4 B per visited voxel-channel (gradient read) + 32 B per
#                   updated voxel-channel (TV term, p, m, v read; p, m, v
#                   written; gradient zeroed) + 32 B per updated k0 voxel (its
#                   BF16 feature record); updated = a nonzero gradient. The
#                   visited and updated counts come from the Adam kernels of
#                   the profiled step (pvdb_march_adam_counts)
RGBNET_FWD_ROW, RGBNET_FWD_RAY, RGBNET_BWD_ROW = 36608.0, 6912.0, 73216.0
# DRAM bytes (read + write) per launch of each stage's kernels at this workload,
# from the ncu captures summarised in profiles/*_bf16_160cube_8192rays.md
# (cold L2; the grids are L2-resident in the live step, so these are the
# bytes a launch pulls from HBM, not the algorithmic bytes above)
NCU_TRAFFIC = {
    "march_fwd": 2.133e6 + 11.115e6,   # k_march_alpha + k_march_chain
    "k0_gather": 9.627e6,              # k_march_k0_x
    "rgbnet_fwd": 14.691e6,            # k_mlp_fwd_tc
    "rgbnet_bwd": 18.388e6,            # k_mlp_bwd_tc
    "march_bwd": 7.145e6,              # k_march_bwd
    "voxel_gather": 11.030e6 + 26.148e6,  # k_group_records + k_voxel_gather
    "tv": 12.608e6,                    # k_tv_terms_c12 (the density grid's k_tv_terms not captured)
    "voxel_adam": 52.651e6 + 3.142e6 + 6.055e6,  # k_vdb_adam_c12 + k_vdb_adam1
}


def touched_leaves(grid):
    import ctypes
    from plenvdb_gb300 import _lib as L
    n = ctypes.c_int64()
    L.call("pvdb_grid_touched_leaves", grid.handle, ctypes.byref(n), L.stream_of())
    return int(n.value)


def adam_counts(ws):
    """Voxels visited and updated by the density and k0 Adam of the last
    profiled step: (density visited, density updated, k0 visited, k0 updated)."""
    import ctypes
    from plenvdb_gb300 import _lib as L
    out = (ctypes.c_int64 * 4)()
    L.call("pvdb_march_adam_counts", ws.h, out, L.stream_of())
    return [int(v) for v in out]


def stage_work(tr, R):
    """(bound, algorithmic units per launch) of each stage for the last step."""
    kept, rows, evaluated = tr.ws.stats()
    C = 12
    feat = getattr(tr, "k0_feature_bytes", 4)  # bytes per gathered k0 feature
    dvis, dupd, kvis, kupd = adam_counts(tr.ws)
    return {
        "march_fwd": ("hbm", evaluated * 36.0),
        "k0_gather": ("hbm", rows * (8 * C * feat + 16.0)),
        "rgbnet_fwd": ("tensor", rows * RGBNET_FWD_ROW + R * RGBNET_FWD_RAY),
        "rgbnet_bwd": ("tensor", rows * RGBNET_BWD_ROW),
        "march_bwd": ("hbm", kept * 120.0),
        "cell_grouping": ("hbm", kept * 32.0),
        "voxel_gather": ("hbm", kept * (64.0 + 8 * (1 + C) * 4.0)),
        "tv": ("hbm", (dvis + kvis * C) * 8.0),
        "voxel_adam": ("hbm", (dvis + kvis * C) * 4.0 + (dupd + kupd * C) * 32.0 + kupd * 32.0),
    }, (kept, rows, evaluated)


def roofline(stage_ms, tr, scfg, R=RAYS):
    """Roofline of the dominant stage: algorithmic bytes (or FLOPs) per launch
    over the stage's CUDA-event time, against the measured peaks."""
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    tflops = float(peaks.get("bf16_tflops", 1900.0))
    work, (kept, rows, evaluated) = stage_work(tr, R)
    table = {}
    for name, ms in stage_ms.items():
        if name not in work or ms <= 0:
            continue
        bound, units = work[name]
        if bound == "hbm":
            ach, peak, unit = units / (ms / 1e3) / 1e9, hbm, "GB/s"
        else:
            ach, peak, unit = units / (ms / 1e3) / 1e12, tflops, "TFLOP/s"
        table[name] = {"bound": bound, "achieved": ach, "unit": unit, "frac": ach / peak,
                       "ms": ms}
    name = max(stage_ms, key=stage_ms.get)
    t = table.get(name)
    src = "MEASURED_PEAKS.json (of measured)" if peaks else "fallback"
    out = {"kernel": name, "bound": t["bound"] if t else "hbm",
           "achieved": t["achieved"] if t else None,
           "peak": (hbm if (not t or t["bound"] == "hbm") else tflops),
           "unit": t["unit"] if t else "GB/s", "frac": t["frac"] if t else None,
           "traffic": NCU_TRAFFIC.get(name) if R == RAYS else None,
           "traffic_source": f"ncu capture, profiles/ (stage {name})" if R == RAYS else None,
           "peak_source": src, "avg_ms": stage_ms[name],
           "kept_samples": kept, "color_rows": rows, "evaluated_samples": evaluated,
           "adam_voxels": dict(zip(["density_visited", "density_updated", "k0_visited",
                                    "k0_updated"], adam_counts(tr.ws))),
           "stages": table}
    return out


def run_render(scfg, cfg, cam, tr, args):
    """800x800 frames along a spiral from a merged index over the trained grids."""
    import torch

    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.renderer import MGRenderer
    from plenvdb_gb300.scene import scene_mask, spiral_poses
    R = scfg.reso
    active = scene_mask(scfg).astype(bool)
    den = tr.density.get_dense_grid().reshape(R, R, R)
    k0 = tr.k0.get_dense_grid().reshape(R, R, R, 12)
    idx = np.zeros((R, R, R), np.int32)
    n = int(active.sum())
    idx[active] = np.arange(1, n + 1, dtype=np.int32)
    den_rows = np.concatenate([[0.0], den[active]]).astype(np.float32)
    col_rows = np.concatenate([np.zeros((1, 12)), k0[active]]).astype(np.float32)
    params = [t.detach().cpu().numpy().T.copy() if t.ndim == 2 else t.detach().cpu().numpy()
              for t in tr.rgbnet_tensors()]
    poses = spiral_poses(max(args.render_frames, 1), cam.radius, -30.0, seed=0)
    res = {}
    for storage, tag in ((0, "fp32"), (1, "bf16")):
        r = MGRenderer(12, 27, 128, 3)
        r.precision = storage  # BF16 features go with the BF16 tensor-core rgbnet
        r.load_data(den_rows, col_rows, idx, n + 1, storage=storage)
        r.load_params(params[0], params[1], params[2], params[3], params[4], params[5])
        r.setScene([R] * 3, cam.K, cfg.xyz_min, cfg.xyz_max)
        r.setKwargs(cam.near, cam.far, cfg.stepdist, cfg.act_shift, cfg.interval,
                    cfg.fast_color_thres, cfg.bg, False, cam.H, cam.W, t_stop=1e-4)
        r.input_a_c2w(poses[0])
        r.render_an_image()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for f in range(args.render_frames):
            r.input_a_c2w(poses[f % len(poses)])
            r.render_an_image()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        img = r.output_an_image()
        res[tag] = {"fps": args.render_frames / dt, "frames": args.render_frames,
                    "mean_rgb": float(img.mean())}
        res[tag + "_last_frame"] = img
    a, b = res.pop("fp32_last_frame"), res.pop("bf16_last_frame")
    res["bf16_vs_fp32_max_abs_rgb"] = float(np.abs(a - b).max())
    res["speedup_bf16"] = res["bf16"]["fps"] / res["fp32"]["fps"]
    res["size"] = f"{cam.W}x{cam.H}"
    res["t_stop"] = 1e-4
    res["timing"] = "wall clock over the frames after one warm-up frame, synchronised"
    return res


def _forward_rgb(ws, dg, kg, net, ro, rd, vd, cfg, precision, batch=RAYS):
    """Composited RGB of many rays through the training forward, in batches."""
    import torch

    from plenvdb_gb300.march import CompositeFn, MarchSample, RgbNetFn, march_params
    p = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                     cfg.interval, cfg.fast_color_thres, cfg.bg)
    dummy = torch.zeros(1, device="cuda")
    out = []
    with torch.no_grad():
        for b in range(0, ro.shape[0], batch):
            sl = slice(b, b + batch)
            w, last, k0, _ = MarchSample.apply(dummy, ws, dg, kg, ro[sl], rd[sl], p)
            rgb = RgbNetFn.apply(k0, vd[sl], ws, 4, precision, *net)
            out.append(CompositeFn.apply(w, rgb, last, ws, cfg.bg).clone())
    return torch.cat(out)


def run_psnr(scfg, cfg, cam, iters, n_views=8):
    """FP32 and BF16 fine-stage training from the same seed (same initial grids,
    rgbnet, ray batches), then PSNR against the ground-truth model on n_views
    held-out 800x800 views, each model evaluated in its own precision."""
    import dataclasses

    import torch

    from plenvdb_gb300.march import MarchWorkspace
    from plenvdb_gb300.scene import (build_grids, random_rays, rays_of_pixels, rgbnet_init,
                                     sphere_poses)
    from plenvdb_gb300.trainer import FineStageTrainer
    t_start = time.perf_counter()
    ws = MarchWorkspace(RAYS, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
    gd, gk = build_grids(scfg, value_seed=4242)
    gt_net = [t.cuda() for t in rgbnet_init(seed=99)]
    # training pool: 64 batches of rays over 100 training views, targets from the
    # ground-truth model
    pool = [torch.from_numpy(a).cuda() for a in random_rays(cam, 64 * RAYS, 100, seed=11)]
    tgt = _forward_rgb(ws, gd, gk, gt_net, *pool, cfg, 0)
    # held-out views (poses not among the training views)
    poses = sphere_poses(n_views, cam.radius, seed=777)
    py, px = np.meshgrid(np.arange(cam.H), np.arange(cam.W), indexing="ij")
    views = []
    for c2w in poses:
        o, d, v = rays_of_pixels(cam, c2w, px.reshape(-1), py.reshape(-1))
        rays = [torch.from_numpy(a).cuda() for a in (o, d, v)]
        views.append((rays, _forward_rgb(ws, gd, gk, gt_net, *rays, cfg, 0)))
    del gd, gk
    gen = torch.Generator(device="cuda")
    res = {"iters": iters, "views": n_views, "size": f"{cam.W}x{cam.H}", "rays_per_iter": RAYS}
    for prec, tag in ((0, "fp32"), (1, "bf16")):
        pcfg = dataclasses.replace(cfg, precision=prec)
        dg, kg = build_grids(scfg)
        tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2), pcfg, max_rays=RAYS)
        gen.manual_seed(5)
        for _ in range(iters):
            idx = torch.randint(0, pool[0].shape[0], (RAYS,), device="cuda", generator=gen)
            tr.step(pool[0][idx], pool[1][idx], pool[2][idx], tgt[idx])
        torch.cuda.synchronize()
        net = [t.contiguous() for t in tr.rgbnet_tensors()]
        ps = []
        for rays, gt in views:
            img = _forward_rgb(ws, dg, kg, net, *rays, cfg, prec)
            mse = float(((img - gt) ** 2).mean())
            ps.append(-10.0 * np.log10(max(mse, 1e-12)))
        res[f"psnr_{tag}"] = float(np.mean(ps))
        res[f"psnr_{tag}_per_view"] = [round(x, 3) for x in ps]
        del tr, dg, kg
    res["delta_db"] = res["psnr_fp32"] - res["psnr_bf16"]
    res["wall_s"] = time.perf_counter() - t_start
    return res


def run_large(args, steps=10, warmup=3):
    """BF16 (and FP32) fine-stage iteration on a 320^3 grid (32 seeded ellipsoids
    plus a thin shell) with 65536 rays per step; targets from a ground-truth
    model of the same scene with other seeded values."""
    import torch

    from plenvdb_gb300.march import MarchWorkspace
    from plenvdb_gb300.scene import (CameraConfig, SceneConfig, build_grids, random_rays,
                                     rgbnet_init, scene_mask)
    from plenvdb_gb300.trainer import FineStageConfig, FineStageTrainer
    R, reso = 65536, 320
    t_start = time.perf_counter()
    scfg = SceneConfig(reso=reso, n_ellipsoids=32, shell=True, seed=0)
    cam = CameraConfig()
    res = {"workload": f"fine-stage iteration, {R} rays, {reso}^3 sparse VDB (32 ellipsoids + "
                       "shell), k0=12, rgbnet 39-128-128-3, TV 1e-4", "rays": R, "reso": reso}
    nb = 2
    rays = [torch.from_numpy(a).cuda() for a in random_rays(cam, nb * R, 100, seed=21)]
    cfg0 = FineStageConfig(reso=reso)
    gws = MarchWorkspace(R, cfg0.xyz_min, cfg0.xyz_max, cfg0.stepdist)
    gd, gk = build_grids(scfg, value_seed=4242)
    tgt = _forward_rgb(gws, gd, gk, [t.cuda() for t in rgbnet_init(seed=99)], *rays, cfg0, 0,
                       batch=R)
    del gd, gk, gws
    res["active_fraction"] = float(scene_mask(scfg).mean())
    for prec, tag in ((1, "bf16"), (0, "fp32")):
        cfg = FineStageConfig(reso=reso, precision=prec)
        dg, kg = build_grids(scfg)
        tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2), cfg, max_rays=R)
        batches = [tuple(t[b * R:(b + 1) * R] for t in (*rays, tgt)) for b in range(nb)]
        for i in range(warmup):
            tr.step(*batches[i % nb])
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for i in range(steps):
            tr.step(*batches[i % nb])
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        kept, rows, evaluated = tr.ws.stats()
        res[tag] = {"it_s": 1e3 / ms, "ms_per_step": ms, "rays_per_s": R * 1e3 / ms,
                    "kept_samples": kept, "color_rows": rows, "evaluated_samples": evaluated,
                    "loss": float(tr.loss.item())}
        if prec == 1:
            # per-stage times and rooflines at this size (grids beyond L2)
            sm = stage_profile(tr, batches, nb, None, None, n=5)
            roof = roofline(sm, tr, scfg, R=R)
            res[tag]["stage_ms"] = sm
            res[tag]["stages"] = roof["stages"]
            res[tag]["adam_voxels"] = roof["adam_voxels"]
            res[tag]["leaf_staging"] = leaf_staging_compare(tr, batches, nb, None, None, sm, n=5)
        del tr, dg, kg
    res["speedup_bf16"] = res["bf16"]["it_s"] / res["fp32"]["it_s"]
    res["timing"] = (f"CUDA events over {steps} steps after {warmup} warm-up steps; inputs "
                     "(2 x 65536 rays) larger than L2 are not the dominant traffic, no flush")
    res["wall_s"] = time.perf_counter() - t_start
    return res


def _cpu_targets(scfg, cfg, ro, rd, vd):
    """Targets of the rays rendered by the oracle from the seeded ground-truth
    model (value seed 4242, rgbnet seed 99), the workload's definition."""
    from oracle import oracle as O
    from plenvdb_gb300.scene import rgbnet_init, scene_dense
    active, dens, k0 = scene_dense(scfg, value_seed=4242)
    R3 = (scfg.reso,) * 3
    og = O.OGridData(R3, dens, active, background=scfg.background)
    ok = O.OGridData(R3, k0, active, background=0.0)
    p = O.march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                       cfg.interval, cfg.fast_color_thres, cfg.bg)
    mlp = O.MLPWeights(*[t.numpy().astype(np.float64) for t in rgbnet_init(seed=99)], c0=12, pe=4)
    out = []
    for b in range(0, ro.shape[0], RAYS):
        om = O.March(og, ok, ro[b:b + RAYS], rd[b:b + RAYS], p, fp32=True)
        out.append(om.composite(om.rgb(mlp, vd[b:b + RAYS]), cfg.bg))
    return np.concatenate(out).astype(np.float32)


def cpu_fine_steps(scfg, cfg, ro, rd, vd, tgt, warmup, steps, budget_s=None):
    """Full 8192-ray fine-stage iterations of the CPU implementation (the
    oracle port, FP32, OpenMP on all host cores) over the workload's batches.
    Returns (seconds per iteration, iterations timed)."""
    from oracle import oracle as O
    from plenvdb_gb300.scene import rgbnet_init, scene_dense
    active, dens, k0 = scene_dense(scfg)
    tr = O.CPUTrainer([scfg.reso] * 3, dens, k0, active, scfg.background,
                      [t.numpy() for t in rgbnet_init(seed=2)])
    p = O.march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                       cfg.interval, cfg.fast_color_thres, cfg.bg)
    nb = ro.shape[0] // RAYS

    def one(i):
        sl = slice((i % nb) * RAYS, (i % nb + 1) * RAYS)
        tr.step(ro[sl], rd[sl], vd[sl], tgt[sl], p)

    for i in range(warmup):
        one(i)
    t0 = time.perf_counter()
    n = 0
    while n < steps:
        one(warmup + n)
        n += 1
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
    return (time.perf_counter() - t0) / n, n


def cpu_density_steps(scfg, cfg, ro, rd, warmup, steps, budget_s=None):
    """The density-only FP32 forward + backward on the CPU (oracle port,
    all host cores), full 8192-ray steps. Returns (seconds per step, steps)."""
    from oracle import oracle as O
    from plenvdb_gb300.scene import rgbnet_init, scene_dense
    active, dens, k0 = scene_dense(scfg)
    tr = O.CPUTrainer([scfg.reso] * 3, dens, k0[..., :3] * 0, active, scfg.background,
                      [t.numpy() for t in rgbnet_init(c0=3, seed=2)])
    p = O.march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                       cfg.interval, cfg.fast_color_thres, cfg.bg)
    tgt = np.random.default_rng(3).random(RAYS).astype(np.float32)
    nb = ro.shape[0] // RAYS

    def one(i):
        sl = slice((i % nb) * RAYS, (i % nb + 1) * RAYS)
        tr.gd[...] = 0.0
        tr.density_step(ro[sl], rd[sl], tgt, p)

    for i in range(warmup):
        one(i)
    t0 = time.perf_counter()
    n = 0
    while n < steps:
        one(warmup + n)
        n += 1
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
    return (time.perf_counter() - t0) / n, n


def cpu_render_fps(scfg, cfg, cam, tr, n_pixels=16384):
    """Merged-VDB render of the CPU implementation (the oracle's restatement of
    MGRenderer's march, FP32, OpenMP) on a bounded sample: n_pixels pixels
    spread over one 800x800 frame of the spiral, time scaled to the frame."""
    from oracle import oracle as O
    from plenvdb_gb300.scene import scene_mask, spiral_poses
    R = scfg.reso
    active = scene_mask(scfg).astype(bool)
    den = tr.density.get_dense_grid().reshape(R, R, R)
    k0 = tr.k0.get_dense_grid().reshape(R, R, R, 12)
    idx = np.zeros((R, R, R), np.int32)
    n = int(active.sum())
    idx[active] = np.arange(1, n + 1, dtype=np.int32)
    den_rows = np.concatenate([[0.0], den[active]]).astype(np.float32)
    col_rows = np.concatenate([np.zeros((1, 12)), k0[active]]).astype(np.float32)
    mlp = O.MLPWeights(*[t.detach().cpu().numpy().astype(np.float64)
                         for t in tr.rgbnet_tensors()], c0=12, pe=4)
    c2w = spiral_poses(1, cam.radius, -30.0, seed=0)[0]
    pix = np.linspace(0, cam.H * cam.W - 1, n_pixels).astype(np.int64)
    args = (idx, den_rows, col_rows, mlp, cam.K, c2w, cfg.xyz_min, cfg.xyz_max, cam.H, cam.W,
            cam.near, cfg.stepdist, cfg.act_shift, cfg.interval, cfg.fast_color_thres, cfg.bg,
            1e-4)
    O.render_pixels(*args, pixels=pix[:256], fp32=True)
    t0 = time.perf_counter()
    O.render_pixels(*args, pixels=pix, fp32=True)
    dt = (time.perf_counter() - t0) * (cam.H * cam.W / n_pixels)
    return {"value": 1.0 / dt, "unit": "FPS", "cores": O.num_threads(), "kind": "port",
            "sample": f"{n_pixels} pixels spread over one {cam.W}x{cam.H} frame, time scaled "
                      "to the frame"}


def cpu_baseline(scfg, cfg, cam, ro, rd, vd, tgt, tr, args):
    """The CPU implementation of the path (oracle port, FP32, OpenMP on all
    host cores) on bounded samples of the same workloads: full 8192-ray
    fine-stage iterations for ~20 s, density-only steps for ~5 s, and the
    render on a pixel sample."""
    from oracle import oracle as O
    dt, n = cpu_fine_steps(scfg, cfg, ro, rd, vd, tgt, warmup=1, steps=100, budget_s=20.0)
    ddt, dn = cpu_density_steps(scfg, cfg, ro, rd, warmup=1, steps=100, budget_s=5.0)
    out = {"value": 1.0 / dt, "unit": "it/s", "cores": O.num_threads(), "kind": "port",
           "sample": f"{n} full {RAYS}-ray fine-stage iterations (about 20 s), the same "
                     "batches and targets as the GPU arm",
           "density_only": {"value": 1.0 / ddt, "unit": "it/s", "rays_per_s": RAYS / ddt,
                            "sample": f"{dn} full {RAYS}-ray density-only steps"}}
    if not args.no_render:
        out["render"] = cpu_render_fps(scfg, cfg, cam, tr)
    return out


def _hbm_peak():
    import json as _json
    try:
        return float(_json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), \
            "MEASURED_PEAKS.json (of measured)"
    except Exception:
        return 6800.0, "fallback"


def _time_op(fn, reps=5, warmup=2):
    """Mean device time (ms) of fn() over reps calls, CUDA events on the
    current stream after warm-up calls."""
    import torch
    st = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        fn()
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def _cpu_ms(fn, budget_s=3.0):
    t0 = time.perf_counter()
    n = 0
    while True:
        fn()
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= 5:
            break
    return (time.perf_counter() - t0) / n * 1e3


def run_lifecycle(scfg, cfg, cam, tr):
    """The steps around the training step at the 160^3 workload: device time
    of each (CUDA events, mean of 5 after 2 warm-up calls), its algorithmic
    bytes and the fraction of the measured HBM bandwidth, and the oracle's CPU
    time on the same input (or a stated sample)."""
    import torch

    from oracle import lifecycle as OL
    from oracle import oracle as O
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300 import lifecycle as LC
    from plenvdb_gb300 import rays as RY
    from plenvdb_gb300.plenvdb import ColorVDB, DensityVDB
    from plenvdb_gb300.scene import scene_mask, sphere_poses
    peak, peak_src = _hbm_peak()
    R = scfg.reso
    nvox = R ** 3
    res = {"peak_gbs": peak, "peak_source": peak_src}

    def entry(ms, nbytes, cpu_ms=None, sample=None, extra=None):
        e = {"ms": ms, "bytes": int(nbytes), "gbs": nbytes / ms / 1e6,
             "frac": nbytes / ms / 1e6 / peak}
        if cpu_ms is not None:
            e["cpu_ms"] = cpu_ms
            e["cpu_sample"] = sample
        e.update(extra or {})
        return e

    mask_np = scene_mask(scfg).astype(bool)
    mask = torch.from_numpy(mask_np).cuda()
    # merged compression (FP16 rows), vdb_compression.py
    n_rows = int(mask_np.sum()) + 1
    ms = _time_op(lambda: LC.merge_compress(tr.density, tr.k0, mask))
    dd = tr.density.get_dense_grid().reshape(R, R, R)
    kd = tr.k0.get_dense_grid().reshape(R, R, R, 12)
    cms = _cpu_ms(lambda: OL.merge(dd, kd, mask_np))
    res["merge_compress"] = entry(ms, nvox * (1 + 4) + (n_rows - 1) * (4 + 48 + 2 + 24), cms,
                                  "the whole grid (numpy, 1 thread)",
                                  {"rows": n_rows, "note": "three mask passes (count, "
                                   "rank+write, the caller's count); bytes count one"})
    # progressive rescaling 80^3 -> 160^3 (scale_volume_grid), density and k0
    half = R // 2
    rng = np.random.default_rng(0)
    for C, name in ((1, "rescale_density"), (12, "rescale_k0")):
        src = DensityVDB([half] * 3, 1) if C == 1 else ColorVDB([half] * 3, C)
        vals = rng.normal(0, 1, half ** 3 * C).astype(np.float32)
        src.copyFromDense(vals)
        dst = DensityVDB([R] * 3, 1) if C == 1 else ColorVDB([R] * 3, C)
        ms = _time_op(lambda: L.call("pvdb_grid_resample", src.handle, dst.handle,
                                     L.stream_of()))
        if C == 1:
            cms = _cpu_ms(lambda: OL.resample(vals.reshape(half, half, half, 1), [R] * 3))
            sample = "the whole grid (numpy, 1 thread)"
        else:
            cms = _cpu_ms(lambda: OL.resample(vals.reshape(half, half, half, C)[..., :1],
                                              [R] * 3)) * C
            sample = "one of the 12 channels (numpy, 1 thread), time x12"
        res[name] = entry(ms, (nvox + half ** 3) * C * 4, cms, sample)
        del src, dst
    # update_occupancy_cache on the 160^3 mask cache
    mc = LC.MaskGrid(mask=mask.clone(), xyz_min=cfg.xyz_min, xyz_max=cfg.xyz_max)
    ms = _time_op(lambda: LC.update_occupancy_cache(mc, tr.density, cfg.act_shift, cfg.interval,
                                                    cfg.fast_color_thres))
    og = O.OGridData((R,) * 3, dd.astype(np.float64), mask_np.astype(np.uint8),
                     background=scfg.background)
    cms = _cpu_ms(lambda: OL.occupancy(0, og, (R,) * 3, cfg.xyz_min, cfg.xyz_max, cfg.act_shift,
                                       cfg.interval, cfg.fast_color_thres, mask=mask_np),
                  budget_s=1.0)
    res["occupancy_update"] = entry(ms, nvox * (4 + 1 + 1), cms,
                                    "the whole grid (trilinear in the C oracle, OpenMP; "
                                    "pooling in numpy)")
    # rays of an 800x800 view, the in-mask-cache hit test and the compaction
    pose = sphere_poses(1, cam.radius, seed=5)[0]
    K = np.asarray(cam.K, np.float64)
    H, W = cam.H, cam.W
    ms = _time_op(lambda: RY.get_rays_of_a_view(H, W, K, pose, False, False, False, False))
    cms = _cpu_ms(lambda: OL.get_rays(H, W, K, pose, False, False, False))
    res["get_rays"] = entry(ms, H * W * 36, cms, "the whole view (numpy, 1 thread)",
                            {"rays_per_s": H * W / ms * 1e3})
    o, d, v = RY.get_rays_of_a_view(H, W, K, pose, False, False, False, False)
    model = {"xyz_min": cfg.xyz_min, "xyz_max": cfg.xyz_max, "voxel_size": cfg.voxel_size}
    ms = _time_op(lambda: RY.hit_coarse_geo(o, d, cam.near, 1e9, cfg.stepsize, mask_cache=mc,
                                            **model))
    on, dn = o.cpu().numpy().reshape(-1, 3), d.cpu().numpy().reshape(-1, 3)
    n_cpu = 20000
    stepdist = float(np.float32(cfg.stepsize) * np.float32(cfg.voxel_size))
    cms = _cpu_ms(lambda: OL.hit_coarse_geo(on[:n_cpu], dn[:n_cpu], cfg.xyz_min, cfg.xyz_max,
                                            cam.near, stepdist, mc.mask.cpu().numpy()),
                  budget_s=2.0) * (H * W / n_cpu)
    hit = RY.hit_coarse_geo(o, d, cam.near, 1e9, cfg.stepsize, mask_cache=mc, **model)
    res["hit_coarse_geo"] = entry(ms, H * W * 25, cms,
                                  f"{n_cpu} of the {H * W} rays (C oracle), time scaled",
                                  {"rays_per_s": H * W / ms * 1e3,
                                   "hit_fraction": float(hit.float().mean())})
    rgb = torch.rand(H * W, 3, device="cuda")
    ms = _time_op(lambda: RY._compact(hit, [o, d, v, rgb], H * W))
    kept = int(hit.sum())
    res["compact_rays"] = entry(ms, H * W + kept * 4 * 12 * 2)
    # voxel_count_views: one view at 200x200 rays (downrate 4)
    ro4 = o[::4, ::4].contiguous()
    rd4 = d[::4, ::4].contiguous()
    ws = [R] * 3
    ms = _time_op(lambda: LC.voxel_count_views(ro4[None], rd4[None], [1], cam.near, 1e9,
                                               cfg.stepsize, ws, cfg.voxel_size, cfg.xyz_min,
                                               cfg.xyz_max), reps=3, warmup=1)
    n_samples = int(np.linalg.norm(np.array(ws) + 1) / cfg.stepsize) + 1
    pts = ro4.shape[0] * ro4.shape[1] * n_samples
    ro_np, rd_np = ro4.cpu().numpy().reshape(-1, 3), rd4.cpu().numpy().reshape(-1, 3)
    n_cpu = 500
    cms = _cpu_ms(lambda: OL.view_weight_sums(ro_np[:n_cpu], rd_np[:n_cpu], ws, cfg.xyz_min,
                                              cfg.xyz_max, cam.near, stepdist, n_samples),
                  budget_s=2.0) * (ro_np.shape[0] / n_cpu)
    res["count_views"] = entry(ms, nvox * 8 * 2 + nvox * 4 * 2, cms,
                               f"{n_cpu} of the {ro_np.shape[0]} rays (numpy), time scaled",
                               {"points_per_s": pts / ms * 1e3, "points": pts,
                                "bound": "atomics: 8 per point"})
    return res


def run_reference(args):
    """The reference arm: the CPU implementation of the path (the oracle port;
    the reference's own implementation of it is CUDA, its CPU-side OpenVDB
    needs TBB/Boost/Blosc, and its NanoVDB harness is built from a tree that
    is not on this machine) on the same workload as the GPU arm: the same
    seeded scene, the same 8 batches of 8192 rays, targets rendered from the
    same ground-truth model (by the oracle). Each step is one full 8192-ray
    FP32 fine-stage iteration on all host cores; then the density-only
    forward + backward, timed the same way."""
    ws_, rank, local = dist_info()
    if rank != 0:
        return
    from oracle import oracle as O
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, random_rays, scene_mask
    from plenvdb_gb300.trainer import FineStageConfig
    t_start = time.perf_counter()
    scfg = SceneConfig(reso=RESO, n_ellipsoids=8, seed=0)
    cfg = FineStageConfig(reso=RESO)
    cam = CameraConfig()
    ro, rd, vd = random_rays(cam, RAYS * N_BATCHES, 100, seed=1)
    tgt = _cpu_targets(scfg, cfg, ro, rd, vd)
    dt, n = cpu_fine_steps(scfg, cfg, ro, rd, vd, tgt, warmup=args.warmup, steps=args.steps)
    ddt, dn = cpu_density_steps(scfg, cfg, ro, rd, warmup=1, steps=min(args.steps, 20))
    val = 1.0 / dt
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": "it/s",
           "n_gpus": ws_, "steps": n, "warmup": args.warmup, "ms_per_step": dt * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "precision": "fp32 (the CPU implementation has no BF16 path)",
           "data": "synthetic: seeded 8-ellipsoid 160^3 scene, 100 seeded 800x800 views, "
                   "targets rendered from a seeded ground-truth grid",
           "config": workload_config(float(scene_mask(scfg).mean())),
           "density_only_it_s": 1.0 / ddt, "density_only_rays_s": RAYS / ddt,
           "cpu_baseline": {"value": val, "unit": "it/s", "cores": O.num_threads(),
                            "kind": "port",
                            "sample": f"each step one full {RAYS}-ray iteration ({n} steps after "
                                      f"{args.warmup} warm-up steps)"},
           "e2e": {"value": val, "unit": "it/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "wall_s": time.perf_counter() - t_start}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.lifecycle_only:
        import torch

        from plenvdb_gb300 import _lib as L
        from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids
        from plenvdb_gb300.trainer import FineStageConfig
        L.load()
        scfg = SceneConfig(reso=RESO, n_ellipsoids=8, seed=0)
        cfg = FineStageConfig(reso=RESO)
        dg, kg = build_grids(scfg)
        grids = type("Grids", (), {"density": dg, "k0": kg})()
        print(json.dumps({"lifecycle": run_lifecycle(scfg, cfg, CameraConfig(), grids)}),
              flush=True)
        torch.cuda.synchronize()
    elif args.large_only:
        import torch

        from plenvdb_gb300 import _lib as L
        L.load()
        print(json.dumps({"large": run_large(args, steps=args.steps, warmup=args.warmup)}),
              flush=True)
        torch.cuda.synchronize()
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
