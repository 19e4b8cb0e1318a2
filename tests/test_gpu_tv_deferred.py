"""Sparse TV in the fused train step: the TV terms computed beside the
per-voxel gradient sums and added by the voxel Adam (the default) give
bitwise the grids, rgbnet parameters and losses of TV added to the gradient
in place before Adam (tv_in_place, the reference's order), over several
steps — graph replays and eager launches, FP32 and BF16, at 160^3 and on the
320^3 scene."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _train(scfg, reso, rays, precision, use_graph, tv_in_place, steps=5, tv_weight=1e-2):
    import torch
    from plenvdb_gb300.scene import CameraConfig, build_grids, random_rays, rgbnet_init
    from plenvdb_gb300.trainer import FineStageConfig, FineStageTrainer
    cfg = FineStageConfig(reso=reso, precision=precision, use_graph=use_graph,
                          tv_in_place=tv_in_place, tv_weight=tv_weight)
    dg, kg = build_grids(scfg)
    tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2), cfg, max_rays=rays)
    ro, rd, vd = random_rays(CameraConfig(), 2 * rays, 100, seed=13)
    tgt = np.random.default_rng(14).random((2 * rays, 3)).astype(np.float32)
    dev = [torch.from_numpy(a).cuda() for a in (ro, rd, vd, tgt)]
    losses = []
    for i in range(steps):
        b = i % 2
        losses.append(float(tr.step(*(t[b * rays:(b + 1) * rays] for t in dev))))
    torch.cuda.synchronize()
    out = (losses, dg.get_dense_grid(device=True).cpu().numpy(),
           kg.get_dense_grid(device=True).cpu().numpy(), tr.params.cpu().numpy())
    del tr, dg, kg
    torch.cuda.empty_cache()
    return out


@pytest.mark.parametrize("reso,precision,use_graph", [(160, 0, False), (160, 1, True),
                                                      (320, 1, True)])
def test_deferred_tv_is_bitwise_in_place_tv(lib, reso, precision, use_graph):
    from plenvdb_gb300.scene import SceneConfig
    scfg = SceneConfig(reso=reso, n_ellipsoids=8 if reso == 160 else 32, shell=reso == 320,
                       seed=0)
    rays = 4096 if reso == 160 else 16384
    a = _train(scfg, reso, rays, precision, use_graph, tv_in_place=False)
    b = _train(scfg, reso, rays, precision, use_graph, tv_in_place=True)
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        np.testing.assert_array_equal(x, y)
    # the TV weight is large enough to move the values: the comparison is not vacuous
    c = _train(scfg, reso, rays, precision, use_graph, tv_in_place=False, tv_weight=0.0)
    assert not np.array_equal(a[1], c[1]) and not np.array_equal(a[2], c[2])
