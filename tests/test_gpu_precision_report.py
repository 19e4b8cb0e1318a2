"""Per-output error of the CUDA path against the FP64 oracle, FP32 and BF16.

One staged iteration (MarchSample -> RgbNetFn -> CompositeFn -> MSE, then the
backward) on a 40^3 scene is compared output by output with the oracle's FP64
forward and backward (dvgo.py:296-370 and the reference kernels' gradients).
Each row reports max |gpu - fp64| and that maximum relative to max |fp64|
(scale-relative), and the assertions hold the FP32 path to 1e-5 (forward) and
1e-4 (gradients) and the BF16 path to the bounds its BF16 rgbnet operands
allow. With PVDB_PRECISION_REPORT=<path> the table is also written as JSON.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RESO = 40


def _err(gpu, ref):
    gpu = np.asarray(gpu, np.float64).reshape(-1)
    ref = np.asarray(ref, np.float64).reshape(-1)
    d = np.abs(gpu - ref)
    scale = max(float(np.abs(ref).max()), 1e-30)
    return {"max_abs": float(d.max()), "rel_to_scale": float(d.max() / scale),
            "scale": scale, "n": int(ref.size)}


@pytest.fixture(scope="module")
def problem(lib):
    from plenvdb_gb300.march import march_params
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, random_rays, scene_dense
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=RESO, n_ellipsoids=5, seed=11)
    cfg = FineStageConfig(reso=RESO)
    ro, rd, vd = random_rays(CameraConfig(), 600, 6, seed=14)
    active, dens, k0 = scene_dense(scfg)
    R3 = (RESO,) * 3
    og = O.OGridData(R3, dens, active, background=scfg.background)
    ok = O.OGridData(R3, k0, active, background=0.0)
    # bg = 1: the composite's alphainv_last * bg term carries gradient too
    op = O.march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                        cfg.interval, cfg.fast_color_thres, 1.0)
    gp = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                      cfg.interval, cfg.fast_color_thres)
    target = np.random.default_rng(2).random((ro.shape[0], 3)).astype(np.float32)
    return dict(scfg=scfg, cfg=cfg, ro=ro, rd=rd, vd=vd, og=og, ok=ok, op=op, gp=gp,
                target=target)


def _gpu_iteration(p, precision):
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import CompositeFn, MarchSample, MarchWorkspace, RgbNetFn
    from plenvdb_gb300.scene import build_grids, rgbnet_init
    cfg = p["cfg"]
    dg, kg = build_grids(p["scfg"])
    dg.zero_grad()
    kg.zero_grad()
    ws = MarchWorkspace(1024, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
    dummy = torch.zeros(1, device="cuda", requires_grad=True)
    ro, rd, vd = (torch.from_numpy(a).cuda() for a in (p["ro"], p["rd"], p["vd"]))
    params = [t.cuda().requires_grad_() for t in rgbnet_init(seed=3)]
    w, last, k0, rid = MarchSample.apply(dummy, ws, dg, kg, ro, rd, p["gp"])
    w.retain_grad()
    last.retain_grad()
    rgb = RgbNetFn.apply(k0, vd, ws, 4, precision, *params)
    rgbm = CompositeFn.apply(w, rgb, last, ws, 1.0)
    tgt = torch.from_numpy(p["target"]).cuda()
    loss = ((rgbm - tgt) ** 2).sum() / tgt.numel()
    loss.backward()
    torch.cuda.synchronize()
    return dict(weight=w.detach().cpu().numpy(), T_last=last.detach().cpu().numpy(),
                k0=k0.detach().cpu().numpy(), rid=rid.cpu().numpy(),
                rgb=rgb.detach().cpu().numpy(), rgb_marched=rgbm.detach().cpu().numpy(),
                g_weight=w.grad.cpu().numpy(), g_T_last=last.grad.cpu().numpy(),
                g_density=dg.get_dense_grid(which=L.WHICH_GRAD),
                g_k0=kg.get_dense_grid(which=L.WHICH_GRAD),
                g_params=[t.grad.cpu().numpy() for t in params])


def _fp64_iteration(p):
    from plenvdb_gb300.scene import rgbnet_init
    om = O.March(p["og"], p["ok"], p["ro"], p["rd"], p["op"], fp32=False)
    net = [t.numpy().astype(np.float64) for t in rgbnet_init(seed=3)]
    mlp = O.MLPWeights(*net, c0=12, pe=4)
    rgb = om.rgb(mlp, p["vd"])
    rgbm = om.composite(rgb, 1.0)
    g_rgbm = 2.0 * (rgbm - p["target"].astype(np.float64)) / p["target"].size
    g_d, g_k, g_params = om.backward(mlp, p["vd"], g_rgbm)
    return om, dict(rgb=rgb, rgb_marched=rgbm, g_density=g_d, g_k0=g_k, g_params=g_params)


def test_per_output_error_against_fp64(problem):
    p = problem
    om, ref = _fp64_iteration(p)
    report = {}
    # BF16: the rgbnet's operands carry 8 mantissa bits; per-voxel k0 gradients
    # also see the ReLU units whose pre-activation flips sign under that
    # rounding, hence the looser gradient bound
    bounds = {0: {"fwd": 1e-5, "grad": 1e-4}, 1: {"fwd": 2e-2, "grad": 1e-1}}
    for precision, tag in ((0, "fp32"), (1, "bf16")):
        g = _gpu_iteration(p, precision)
        if g["rgb"].shape[0] != om.M or not np.array_equal(g["rid"], om.ray_id):
            pytest.skip("a threshold decision differs between FP32 and FP64 on this draw")
        rows = {
            "sample weight": _err(g["weight"], om.weight),
            "alphainv_last (T)": _err(g["T_last"], om.T_last),
            "k0 rows": _err(g["k0"], om.k0),
            "rgb (rgbnet)": _err(g["rgb"], ref["rgb"]),
            "rgb_marched": _err(g["rgb_marched"], ref["rgb_marched"]),
            "grad density grid": _err(g["g_density"], ref["g_density"]),
            "grad k0 grid": _err(g["g_k0"], ref["g_k0"]),
        }
        for name, a, b in zip(("w0", "b0", "w1", "b1", "w2", "b2"), g["g_params"],
                              ref["g_params"]):
            rows[f"grad rgbnet {name}"] = _err(a, b)
        report[tag] = rows
    out = os.environ.get("PVDB_PRECISION_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
    for precision, tag in ((0, "fp32"), (1, "bf16")):
        b = bounds[precision]
        for name, e in report[tag].items():
            lim = b["grad"] if name.startswith("grad") else b["fwd"]
            if name in ("sample weight", "alphainv_last (T)", "k0 rows"):
                lim = 1e-5  # the sample stage is FP32 in both precisions
            assert e["rel_to_scale"] <= lim, (tag, name, e)
