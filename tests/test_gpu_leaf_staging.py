"""Leaf staging of the forward's density pass (pvdb_march_set_leaf_staging:
the density leaves of a ray's evaluated samples copied into shared memory by
1-D bulk copies, up to 24 per ray) gives bitwise the results of the default
pass — on the 160^3 bench scene with its 8192-ray batch, on a 1024-ray subset
of the 320^3 scene (rays crossing more leaves than the staging slots), and
through the fused BF16 train step. A copy wait that runs out (test hook: the
first block issues no copies) reports PVDB_ERR_TIMEOUT and still gives the
same values, read from global memory."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(reso, n_ell, shell, n_rays, ray_seed, subset=None):
    from plenvdb_gb300.march import march_params
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=reso, n_ellipsoids=n_ell, shell=shell, seed=0)
    cfg = FineStageConfig(reso=reso)
    ro, rd, vd = random_rays(CameraConfig(), n_rays, 100, seed=ray_seed)
    if subset is not None:
        pick = np.random.default_rng(5).choice(n_rays, subset, replace=False)
        ro, rd, vd = ro[pick], rd[pick], vd[pick]
    dg, kg = build_grids(scfg)
    gp = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                      cfg.interval, cfg.fast_color_thres)
    return dict(scfg=scfg, cfg=cfg, ro=ro, rd=rd, vd=vd, dg=dg, kg=kg, gp=gp)


def _forward(s, staging):
    import torch
    from plenvdb_gb300.march import MarchSample, MarchWorkspace
    ws = MarchWorkspace(s["ro"].shape[0], s["cfg"].xyz_min, s["cfg"].xyz_max,
                        s["cfg"].stepdist, leaf_staging=staging)
    dummy = torch.zeros(1, device="cuda", requires_grad=True)
    w, last, k0, rid = MarchSample.apply(dummy, ws, s["dg"], s["kg"],
                                         torch.from_numpy(s["ro"]).cuda(),
                                         torch.from_numpy(s["rd"]).cuda(), s["gp"])
    torch.cuda.synchronize()
    out = [t.detach().cpu().numpy() for t in (w, last, k0, rid)]
    return ws, out + [np.array(ws.stats())]


@pytest.mark.parametrize("which", ["bench_160", "large_320_subset"])
def test_staged_density_pass_is_bitwise_the_default(lib, which):
    s = (_scene(160, 8, False, 8192, 1) if which == "bench_160"
         else _scene(320, 32, True, 2 * 65536, 21, subset=1024))
    _, a = _forward(s, False)
    _, b = _forward(s, True)
    assert a[0].size > 1000
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_staging_copy_wait_reports_timeout_and_keeps_values(lib):
    from plenvdb_gb300 import _lib as L
    s = _scene(160, 8, False, 512, 4)
    _, ref = _forward(s, False)
    L.call("pvdb_debug_wait_limit", 1 << 16, 2)
    try:
        ws, got = _forward_unchecked(s)
    finally:
        L.call("pvdb_debug_wait_limit", 0, 0)
    tk, tr = C.c_int64(), C.c_int64()
    rc = L.load().pvdb_march_totals(ws.h, C.byref(tk), C.byref(tr), L.stream_of())
    assert rc == L.PVDB_ERR_TIMEOUT, (rc, L.last_error())
    assert "leaf-staging" in L.last_error()
    for x, y in zip(ref[:4], got):
        np.testing.assert_array_equal(x, y)
    # the context is usable and the staged pass is clean again
    _, again = _forward(s, True)
    for x, y in zip(ref, again):
        np.testing.assert_array_equal(x, y)


def _forward_unchecked(s):
    """The staged forward through the C ABI, without the status check that
    MarchSample makes (the timeout is read afterwards)."""
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import MarchWorkspace
    R = s["ro"].shape[0]
    ws = MarchWorkspace(R, s["cfg"].xyz_min, s["cfg"].xyz_max, s["cfg"].stepdist,
                        leaf_staging=True)
    tro, trd = torch.from_numpy(s["ro"]).cuda(), torch.from_numpy(s["rd"]).cuda()
    L.call("pvdb_march_forward", ws.h, s["dg"].handle, s["kg"].handle, L.ptr(tro), L.ptr(trd),
           R, C.byref(s["gp"]), None, None, L.stream_of())
    torch.cuda.synchronize()
    ws.n_rays = R
    tk, tr = C.c_int64(), C.c_int64()
    L.load().pvdb_march_totals(ws.h, C.byref(tk), C.byref(tr), L.stream_of())
    rows = ws.rows(tr.value, 12)
    return ws, [rows[k].cpu().numpy() for k in ("weight", "alphainv_last", "k0", "ray_id")]


def test_fused_train_step_with_staging_is_bitwise_the_default(lib):
    import torch
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays, rgbnet_init
    from plenvdb_gb300.trainer import FineStageConfig, FineStageTrainer
    scfg = SceneConfig(reso=160, n_ellipsoids=8, seed=0)
    ro, rd, vd = random_rays(CameraConfig(), 4096, 100, seed=7)
    tgt = np.random.default_rng(8).random((4096, 3)).astype(np.float32)
    batch = [torch.from_numpy(a).cuda() for a in (ro, rd, vd, tgt)]
    res = []
    for staging in (False, True):
        cfg = FineStageConfig(reso=160, precision=1, use_graph=True, leaf_staging=staging)
        dg, kg = build_grids(scfg)
        tr = FineStageTrainer(dg, kg, rgbnet_init(seed=2), cfg, max_rays=4096)
        losses = [float(tr.step(*batch)) for _ in range(4)]
        torch.cuda.synchronize()
        res.append((losses, dg.get_dense_grid(device=True).cpu().numpy(),
                    kg.get_dense_grid(device=True).cpu().numpy(), tr.params.cpu().numpy()))
    assert res[0][0] == res[1][0]
    for x, y in zip(res[0][1:], res[1][1:]):
        np.testing.assert_array_equal(x, y)
