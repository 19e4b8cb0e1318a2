"""The BF16 train step gathers 12-channel k0 features from the grid's BF16
shadow, which the voxel Adam keeps current beside the FP32 master values.

A run whose shadow is maintained by Adam (graph replay) must equal, bit for
bit, a run that rebuilds the shadow from the FP32 master values before every
step (the k0 grid marked as written from outside each time, eager launches):
both gather round-to-nearest BF16 copies of the same FP32 values. The FP32
plain method never reads the shadow."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_adam_maintained_shadow_equals_rebuilt_shadow(lib):
    import dataclasses

    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.scene import (CameraConfig, SceneConfig, build_grids, random_rays,
                                     rgbnet_init)
    from plenvdb_gb300.trainer import FineStageConfig, FineStageTrainer
    scfg = SceneConfig(reso=40, n_ellipsoids=5, seed=11)
    cfg = FineStageConfig(reso=40, precision=1, use_graph=True)
    ro, rd, vd = random_rays(CameraConfig(), 2048, 6, seed=4)
    g = torch.Generator().manual_seed(9)
    batches = []
    for b in range(3):
        perm = torch.randperm(2048, generator=g)[:700]
        batches.append(tuple(torch.from_numpy(a)[perm].contiguous().cuda() for a in (ro, rd, vd))
                       + (torch.rand(700, 3, generator=g).cuda(),))
    runs = []
    for rebuild in (False, True):
        dg, kg = build_grids(scfg)
        tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2),
                              dataclasses.replace(cfg, use_graph=not rebuild), max_rays=1024)
        assert tr.k0_feature_bytes == 2
        losses = []
        for i in range(12):
            if rebuild:
                kg.mark_written(L.WHICH_DATA)  # the next step rebuilds the shadow
            losses.append(float(tr.step(*batches[i % 3])))
        runs.append((losses, dg.get_dense_grid(), kg.get_dense_grid(), tr.params.cpu().numpy()))
    (la, da, ka, pa), (lb, db, kb, pb) = runs
    assert la == lb
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(pa, pb)
    assert la[-1] < la[0]
