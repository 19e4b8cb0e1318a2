"""BF16 tensor-core (tcgen05) rgbnet against the FP32 SIMT rgbnet and an FP64
torch reference. BF16 operands with FP32 accumulation: the tolerance is the
BF16 rounding of activations and weights (about 3 significant digits)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rows(lib):
    import torch
    from plenvdb_gb300.march import MarchSample, MarchWorkspace, march_params
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=64, n_ellipsoids=6, seed=5)
    cfg = FineStageConfig(reso=64)
    dg, kg = build_grids(scfg)
    ro, rd, vd = random_rays(CameraConfig(), 2000, 8, seed=2)
    ws = MarchWorkspace(2048, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
    p = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                     cfg.interval, cfg.fast_color_thres)
    dummy = torch.zeros(1, device="cuda")
    w, last, k0, rid = MarchSample.apply(dummy, ws, dg, kg, torch.from_numpy(ro).cuda(),
                                         torch.from_numpy(rd).cuda(), p)
    return ws, k0, rid, torch.from_numpy(vd).cuda(), (dg, kg)


def _torch_rgb(k0, rid, vd, params):
    import torch
    P = [t.double() for t in params]
    v = vd.double()
    freq = torch.tensor([1.0, 2.0, 4.0, 8.0], dtype=torch.float64, device="cuda")
    emb = (v.unsqueeze(-1) * freq).flatten(-2)
    pe = torch.cat([v, emb.sin(), emb.cos()], -1)[rid.long()]
    x = torch.cat([k0.double(), pe], -1)
    h = torch.relu(x @ P[0].T + P[1])
    h = torch.relu(h @ P[2].T + P[3])
    return torch.sigmoid(h @ P[4].T + P[5])


@pytest.mark.parametrize("seed", [3, 4])
def test_tc_forward_matches_fp32_and_fp64(rows, seed):
    import torch
    from plenvdb_gb300.march import RgbNetFn
    from plenvdb_gb300.scene import rgbnet_init
    ws, k0, rid, vd, _ = rows
    params = [t.cuda() for t in rgbnet_init(seed=seed)]
    # larger k0 features so layer 0 matters
    k0s = (k0 * 10).contiguous()
    with torch.no_grad():
        rgb32 = RgbNetFn.apply(k0s, vd, ws, 4, 0, *params)
        rgb16 = RgbNetFn.apply(k0s, vd, ws, 4, 1, *params)
        ref = _torch_rgb(k0s, rid, vd, params)
    assert k0.shape[0] > 5000
    err16 = (rgb16.double() - ref).abs()
    err32 = (rgb32.double() - ref).abs()
    assert err32.max().item() < 1e-5
    assert err16.max().item() < 2e-2, err16.max().item()
    assert err16.mean().item() < 2e-3, err16.mean().item()
    # every row was computed (no untouched output)
    assert torch.isfinite(rgb16).all()


def test_tc_forward_deterministic(rows):
    import torch
    from plenvdb_gb300.march import RgbNetFn
    from plenvdb_gb300.scene import rgbnet_init
    ws, k0, rid, vd, _ = rows
    params = [t.cuda() for t in rgbnet_init(seed=1)]
    with torch.no_grad():
        a = RgbNetFn.apply(k0, vd, ws, 4, 1, *params)
        b = RgbNetFn.apply(k0, vd, ws, 4, 1, *params)
    assert torch.equal(a, b)


def test_render_bf16_close_to_fp32(lib):
    import torch
    from plenvdb_gb300.renderer import MGRenderer
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, scene_dense, rgbnet_init, spiral_poses
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=64, n_ellipsoids=6, seed=5)
    cfg = FineStageConfig(reso=64)
    cam = CameraConfig(H=200, W=200, focal=277.8)
    active, dens, k0 = scene_dense(scfg)
    act = active.astype(bool)
    n = int(act.sum())
    idx = np.zeros(act.shape, np.int32)
    idx[act] = np.arange(1, n + 1)
    den = np.concatenate([[0.0], dens[act]]).astype(np.float32)
    col = np.concatenate([np.zeros((1, 12)), k0[act] * 10]).astype(np.float32)
    params = [t.numpy().T.copy() if t.ndim == 2 else t.numpy() for t in rgbnet_init(seed=2)]
    imgs = {}
    for prec in (0, 1):
        r = MGRenderer(12, 27, 128, 3)
        r.precision = prec
        r.load_data(den, col, idx, n + 1)
        r.load_params(*params)
        r.setScene([64] * 3, cam.K, cfg.xyz_min, cfg.xyz_max)
        r.setKwargs(cam.near, cam.far, cfg.stepdist, cfg.act_shift, cfg.interval,
                    cfg.fast_color_thres, 1.0, False, cam.H, cam.W)
        r.input_a_c2w(spiral_poses(1, cam.radius, -30.0)[0])
        r.render_an_image()
        imgs[prec] = r.output_an_image().reshape(cam.H, cam.W, 3)
    d = np.abs(imgs[0] - imgs[1])
    assert d.max() < 2e-2 and d.mean() < 1e-3, (d.max(), d.mean())
    assert np.abs(imgs[0] - 1.0).max() > 0.1  # the scene is visible
