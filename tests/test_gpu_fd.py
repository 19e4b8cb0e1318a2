"""Gradients of the CUDA path (FP32 plain method) against FP64 central finite
differences of the oracle's loss at the fine-stage configuration: the 160^3
bench scene (8 seeded ellipsoids), a seeded 8192-ray batch, 64 voxel values
(48 density voxels and 16 k0 voxel-channels with the largest gradients),
eps = 1e-4.

Loss: MSE of the composited colour (bg = 1) against a seeded target, through
the whole forward (sample, raw2alpha, alpha2weight, thresholds, k0, rgbnet,
composite). A voxel value only changes rays that sample a trilinear cell it
is a corner of, so each difference quotient is evaluated on those rays (a
one-cell margin around the voxel's cells; the loss keeps the full batch's
normalisation), with the value perturbed in place in the oracle's grid.

A central difference is only meaningful where no threshold decision
(alpha / weight > thres, T < t_stop) flips inside [v - eps, v + eps]; such
values are recognised by their difference quotient changing between eps and
eps / 2, and are left out (at most a few of the 64)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RESO = 160
N_RAYS = 8192
EPS = 1e-4


@pytest.fixture(scope="module")
def problem(lib):
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, random_rays, scene_dense
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=RESO, n_ellipsoids=8, seed=0)
    cfg = FineStageConfig(reso=RESO)
    ro, rd, vd = random_rays(CameraConfig(), N_RAYS, 100, seed=23)
    active, dens, k0 = scene_dense(scfg)
    R3 = (RESO,) * 3
    og = O.OGridData(R3, dens, active, background=scfg.background)
    ok = O.OGridData(R3, k0, active, background=0.0)
    op = O.march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                        cfg.interval, cfg.fast_color_thres, 1.0)
    target = np.random.default_rng(4).random((N_RAYS, 3))
    # every evaluated sample's trilinear cell, for the rays-per-voxel lookup
    pts, outb, rid, _ = O.ray_points(ro, rd, op)
    keep = ~outb
    mn = np.float32(cfg.xyz_min[0])
    ext = np.float32(cfg.xyz_max[0]) - mn
    idx = ((pts[keep] - mn) / ext) * np.float32(RESO - 1)
    cells = np.floor(idx).astype(np.int32)
    return dict(scfg=scfg, cfg=cfg, ro=ro, rd=rd, vd=vd, active=active, dens=dens, k0=k0,
                og=og, ok=ok, op=op, target=target, cells=cells, cell_ray=rid[keep])


def _gpu_grads(p):
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import CompositeFn, MarchSample, MarchWorkspace, RgbNetFn, march_params
    from plenvdb_gb300.scene import build_grids, rgbnet_init
    cfg = p["cfg"]
    dg, kg = build_grids(p["scfg"])
    dg.zero_grad()
    kg.zero_grad()
    gp = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                      cfg.interval, cfg.fast_color_thres)
    ws = MarchWorkspace(N_RAYS, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
    dummy = torch.zeros(1, device="cuda", requires_grad=True)
    ro, rd, vd = (torch.from_numpy(a).cuda() for a in (p["ro"], p["rd"], p["vd"]))
    params = [t.cuda() for t in rgbnet_init(seed=3)]
    w, last, k0, rid = MarchSample.apply(dummy, ws, dg, kg, ro, rd, gp)
    rgb = RgbNetFn.apply(k0, vd, ws, 4, 0, *params)
    rgbm = CompositeFn.apply(w, rgb, last, ws, 1.0)
    tgt = torch.from_numpy(p["target"]).float().cuda()
    loss = ((rgbm - tgt) ** 2).sum() / tgt.numel()
    loss.backward()
    torch.cuda.synchronize()
    R3 = (RESO,) * 3
    return (dg.get_dense_grid(which=L.WHICH_GRAD).reshape(R3).astype(np.float64),
            kg.get_dense_grid(which=L.WHICH_GRAD).reshape(R3 + (12,)).astype(np.float64))


def _rays_near(p, v):
    """Rays with an evaluated sample in a cell within one cell of the voxel's
    eight trilinear cells."""
    c = p["cells"]
    near = np.all((c >= np.array(v) - 2) & (c <= np.array(v) + 1), axis=1)
    return np.unique(p["cell_ray"][near])


def _loss64(p, rays):
    from plenvdb_gb300.scene import rgbnet_init
    om = O.March(p["og"], p["ok"], p["ro"][rays], p["rd"][rays], p["op"], fp32=False)
    net = [t.numpy().astype(np.float64) for t in rgbnet_init(seed=3)]
    mlp = O.MLPWeights(*net, c0=12, pe=4)
    rgbm = om.composite(om.rgb(mlp, p["vd"][rays]), 1.0)
    return float(((rgbm - p["target"][rays]) ** 2).sum() / p["target"].size)


def _central(p, which, index, eps):
    g = p["og"] if which == "density" else p["ok"]
    vox = index[:3]
    rays = _rays_near(p, vox)
    P = g.pad
    flat = ((vox[0] * P[1] + vox[1]) * P[2] + vox[2]) * g.C + (index[3] if which == "k0" else 0)
    base = g.p_values[flat]
    try:
        g.p_values[flat] = base + eps
        lp = _loss64(p, rays)
        g.p_values[flat] = base - eps
        lm = _loss64(p, rays)
    finally:
        g.p_values[flat] = base
    return (lp - lm) / (2 * eps)


def test_gradients_match_fp64_central_differences(problem):
    p = problem
    gd, gk = _gpu_grads(p)
    act = p["active"].astype(bool)
    # 48 density voxels and 16 k0 voxel-channels with the largest gradients
    d_idx = np.argsort(-np.abs(np.where(act, gd, 0.0)).ravel())[:48]
    k_idx = np.argsort(-np.abs(np.where(act[..., None], gk, 0.0)).ravel())[:16]
    cases = [("density", tuple(int(x) for x in np.unravel_index(i, gd.shape)), gd)
             for i in d_idx]
    cases += [("k0", tuple(int(x) for x in np.unravel_index(i, gk.shape)), gk) for i in k_idx]
    checked = 0
    worst = 0.0
    for which, index, g in cases:
        fd = _central(p, which, index, EPS)
        fd2 = _central(p, which, index, EPS / 2)
        if abs(fd - fd2) > 1e-3 * max(abs(fd), abs(fd2), 1e-12):
            continue  # a threshold decision flips within the step
        checked += 1
        scale = np.abs(g).max()
        err = abs(g[index] - fd)
        worst = max(worst, err / max(abs(fd), 1e-3 * scale))
        assert err <= 1e-4 * abs(fd) + 1e-6 * scale, (which, index, g[index], fd)
    assert checked >= 56, f"only {checked} of 64 values had a smooth central difference"
    print(f"checked {checked} of 64; worst relative error {worst:.2e}")
