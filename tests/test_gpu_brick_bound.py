"""The density grid's brick bounds, which let the march skip the trilinear of
samples whose alpha cannot pass the threshold, stay upper bounds while voxel
Adam changes the density: after fused training steps (BF16, graph replays;
voxel Adam raises the bounds of the voxels that grew, a warp's raises merged
per brick), a forward gives bitwise the same weights, transmittance, k0 rows
and ray ids as a forward after the bounds were rebuilt from the values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("reso,n_ell,shell,rays", [(160, 8, False, 8192), (320, 32, True, 16384)])
def test_bounds_after_training_match_rebuilt_bounds(lib, reso, n_ell, shell, rays):
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import MarchSample, MarchWorkspace, march_params
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays, rgbnet_init
    from plenvdb_gb300.trainer import FineStageConfig, FineStageTrainer
    scfg = SceneConfig(reso=reso, n_ellipsoids=n_ell, shell=shell, seed=0)
    cfg = FineStageConfig(reso=reso, precision=1, use_graph=True, lr_density=0.5)
    dg, kg = build_grids(scfg)
    tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2), cfg, max_rays=rays)
    ro, rd, vd = random_rays(CameraConfig(), 2 * rays, 100, seed=9)
    tgt = np.random.default_rng(10).random((2 * rays, 3)).astype(np.float32)
    dev = [torch.from_numpy(a).cuda() for a in (ro, rd, vd, tgt)]
    for i in range(8):
        b = i % 2
        tr.step(*(t[b * rays:(b + 1) * rays] for t in dev))
    torch.cuda.synchronize()
    gp = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                      cfg.interval, cfg.fast_color_thres)
    pro, prd, _ = random_rays(CameraConfig(), rays, 100, seed=31)
    pro, prd = torch.from_numpy(pro).cuda(), torch.from_numpy(prd).cuda()

    def forward():
        ws = MarchWorkspace(rays, cfg.xyz_min, cfg.xyz_max, cfg.stepdist)
        dummy = torch.zeros(1, device="cuda", requires_grad=True)
        out = MarchSample.apply(dummy, ws, dg, kg, pro, prd, gp)
        torch.cuda.synchronize()
        return [t.detach().cpu().numpy() for t in out], ws.stats()

    a, sa = forward()
    dg.mark_written(L.WHICH_DATA)  # the bounds are rebuilt from the values at the next march
    b, sb = forward()
    assert a[0].size > 1000
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert sa[:2] == sb[:2]
    # the rebuilt bounds are tight: they never let more samples through
    assert sb[2] <= sa[2]
