"""The DVGO schedule around the training step on the GPU (lifecycle.cu,
rays.cu through include/pvdb.h) against the oracle (oracle/lifecycle.py) and
the reference's own outputs (tests/golden/lifecycle_golden.npz):

* merged compression: index and FP16/FP32 rows bit-exact, empty / full /
  ragged masks, unaligned mask buffers, a wrong row count refused;
* stable compaction of ray arrays;
* rescaling (align_corners trilinear) bit-exact, up and down, 1 and 12
  channels, sparse sources (background outside leaves);
* the three mask-cache builds: exact except voxels sitting on the threshold;
* near-camera masking exact; per-view voxel counts exact except voxels whose
  weight sum is within 1e-4 of 1;
* rays (all flag combinations, NDC, random jitter) and hit_coarse_geo exact;
  the in-mask-cache training-ray gatherer against the reference composition;
* merged files round trip into MGRenderer; trainer checkpoint/resume is
  bitwise identical to an uninterrupted run."""
import os

import numpy as np
import pytest

from oracle import lifecycle as OL
from oracle import oracle as O

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "lifecycle_golden.npz"))


def _sparse(R, seed, C=1, bg=-10.0, p=0.3):
    """A sparse grid (leaves holding an active voxel) with seeded values; the
    dense view the oracle reads (background outside leaves)."""
    from plenvdb_gb300.plenvdb import ColorVDB, DensityVDB
    rng = np.random.default_rng(seed)
    active = (rng.random(R) < p).astype(np.uint8)
    active[: R[0] // 3, : R[1] // 2, :] = 0  # whole empty leaves
    vals = rng.normal(0, 2, R + ((C,) if C > 1 else ())).astype(np.float32)
    g = (DensityVDB.from_mask(list(R), active, background=bg) if C == 1 else
         ColorVDB.from_mask(list(R), active, background=bg, n=C))
    g.copyFromDense(vals.reshape(-1))
    dense = g.get_dense_grid().reshape(R + ((C,) if C > 1 else ()))
    return g, dense, active


# ------------------------------------------------------------------ merge
@pytest.mark.parametrize("kind", ["random", "empty", "full"])
def test_merge_bit_exact(lib, kind):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    R = (37, 21, 29)  # voxel count not a multiple of the 16-byte chunks
    dg, dd, _ = _sparse(R, 1)
    kg, kd, _ = _sparse(R, 2, C=12, bg=0.0)
    rng = np.random.default_rng(3)
    mask = {"random": rng.random(R) < 0.4, "empty": np.zeros(R, bool),
            "full": np.ones(R, bool)}[kind]
    for dtype, npdt in (("float16", np.float16), ("float32", np.float32)):
        out = LC.merge_compress(dg, kg, torch.from_numpy(mask).cuda(), row_dtype=dtype)
        idx, den, col = OL.merge(dd, kd, mask, dtype=npdt)
        np.testing.assert_array_equal(out["index"].cpu().numpy(), idx)
        assert out["N"] == int(mask.sum()) + 1
        if npdt is np.float16:
            np.testing.assert_array_equal(out["den"].cpu().numpy().view(np.uint16),
                                          den.view(np.uint16))
            np.testing.assert_array_equal(out["col"].cpu().numpy().view(np.uint16),
                                          col.view(np.uint16))
        else:
            np.testing.assert_array_equal(out["den"].cpu().numpy(), den)
            np.testing.assert_array_equal(out["col"].cpu().numpy(), col)


def test_merge_reference_golden_and_unaligned(lib, gold):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    from plenvdb_gb300.plenvdb import ColorVDB, DensityVDB
    mask = gold["merge_mask"]
    R = list(mask.shape)
    dg = DensityVDB(R, 1)
    kg = ColorVDB(R, 12)
    dg.copyFromDense(gold["merge_den"].reshape(-1))
    kg.copyFromDense(gold["merge_col"].reshape(-1))
    # mask bytes at an odd address: the byte-wise path
    buf = torch.zeros(mask.size + 1, dtype=torch.uint8, device="cuda")
    buf[1:] = torch.from_numpy(mask.reshape(-1).astype(np.uint8)).cuda()
    out = LC.merge_compress(dg, kg, buf[1:].view(mask.shape))
    np.testing.assert_array_equal(out["index"].cpu().numpy(), gold["merge_idxs"].astype(np.int32))
    np.testing.assert_array_equal(out["den"].cpu().numpy().view(np.uint16),
                                  gold["merge_den_rows"].view(np.uint16))
    np.testing.assert_array_equal(out["col"].cpu().numpy().view(np.uint16),
                                  gold["merge_col_rows"].view(np.uint16))


def test_merge_refuses_wrong_row_count(lib):
    import torch
    from plenvdb_gb300 import _lib as L
    dg, _, _ = _sparse((16, 16, 16), 4)
    mask = torch.ones(16, 16, 16, dtype=torch.uint8, device="cuda")
    index = torch.full((16 ** 3,), -7, dtype=torch.int32, device="cuda")
    den = torch.zeros(10, device="cuda")
    with pytest.raises(L.PvdbError, match="n_rows"):
        L.call("pvdb_merge_build", dg.handle, None, L.ptr(mask), L.ptr(index), L.ptr(den), None,
               10, 0, None)
    assert int(index.min()) == -7  # nothing was written


def test_compact_rows_stable(lib):
    import torch
    from plenvdb_gb300.rays import _compact
    rng = np.random.default_rng(5)
    n = 100003
    keep = rng.random(n) < 0.37
    arrs = [rng.normal(size=(n, 3)).astype(np.float32) for _ in range(4)]
    got, k = _compact(torch.from_numpy(keep).cuda(), [torch.from_numpy(a).cuda() for a in arrs], n)
    assert k == int(keep.sum())
    for g, a in zip(got, arrs):
        np.testing.assert_array_equal(g.cpu().numpy(), a[keep])


# --------------------------------------------------------------- rescale
@pytest.mark.parametrize("src,dst,C", [((20, 17, 23), (41, 33, 45), 1),
                                       ((24, 30, 19), (13, 40, 19), 12),
                                       ((9, 9, 9), (1, 5, 2), 1)])
def test_resample_bit_exact(lib, src, dst, C):
    from plenvdb_gb300 import lifecycle as LC
    g, dense, _ = _sparse(src, 6, C=C, bg=-10.0 if C == 1 else 0.0)
    new = LC.scale_volume_grid(g, dst)
    got = new.get_dense_grid().reshape(dst + ((C,) if C > 1 else ()))
    ref = OL.resample(dense.reshape(src + (C,)), dst).reshape(got.shape)
    np.testing.assert_array_equal(got, ref)
    assert new.info()[3] == int(np.prod(dst))  # dense and all active, as the reference


def test_resample_reference_golden(lib, gold):
    from plenvdb_gb300 import lifecycle as LC
    from plenvdb_gb300.plenvdb import ColorVDB, DensityVDB
    for n in range(2):
        src = gold[f"scale{n}_src"]
        C = src.shape[-1]
        g = DensityVDB(list(src.shape[:3]), 1) if C == 1 else ColorVDB(list(src.shape[:3]), C)
        g.copyFromDense(src.reshape(-1))
        new = LC.scale_volume_grid(g, [int(v) for v in gold[f"scale{n}_dst"]])
        np.testing.assert_array_equal(new.get_dense_grid(), gold[f"scale{n}_out"].reshape(-1))


# ------------------------------------------------------------- occupancy
def _occ_dense(gold):
    from plenvdb_gb300.plenvdb import DensityVDB
    dens = gold["occ_dens"]
    g = DensityVDB(list(dens.shape), 1)
    g.copyFromDense(dens.reshape(-1))
    og = O.OGridData(dens.shape, dens.astype(np.float64), np.ones(dens.shape, np.uint8))
    return g, og


def _assert_mask(got, margin, ref, thres):
    diff = got != ref
    near = np.abs(margin.astype(np.float64) - thres) <= 1e-5 * thres
    assert not (diff & ~near).any(), f"{int((diff & ~near).sum())} voxels differ"


def test_occupancy_modes_against_reference(lib, gold):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    g, og = _occ_dense(gold)
    mn, mx = gold["occ_box"]
    shift, interval, thres = (float(v) for v in gold["occ_params"])
    old = gold["occ_old"]
    # mode 0 (update_occupancy_cache), on a mask cache of another shape
    mc = LC.MaskGrid(mask=torch.from_numpy(old.copy()).cuda(), xyz_min=mn, xyz_max=mx)
    LC.update_occupancy_cache(mc, g, shift, interval, thres)
    _, margin = OL.occupancy(0, og, old.shape, mn, mx, shift, interval, thres, mask=old)
    _assert_mask(mc.mask.cpu().numpy().astype(bool), margin, gold["occ_mode0"], thres)
    # mode 1 (the rebuild after rescaling)
    mc_old = LC.MaskGrid(mask=torch.from_numpy(old.copy()).cuda(), xyz_min=mn, xyz_max=mx)
    new = LC.rescaled_mask_cache(mc_old, g, mn, mx, shift, interval, thres)
    _, margin = OL.occupancy(1, og, og.reso, mn, mx, shift, interval, thres, old_mask=old)
    _assert_mask(new.mask.cpu().numpy().astype(bool), margin, gold["occ_mode1"], thres)
    # mode 2 (MaskGrid from a checkpoint's density)
    m2 = LC.mask_from_density(g, shift, interval, thres, mn, mx)
    _, margin = OL.occupancy(2, og, og.reso, mn, mx, shift, interval, thres)
    _assert_mask(m2.cpu().numpy().astype(bool), margin, gold["occ_mode2"], thres)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_occupancy_sparse_grid_against_oracle(lib, mode):
    import torch
    from plenvdb_gb300 import _lib as L
    R = (30, 26, 35)
    g, dense, active = _sparse(R, 8, bg=-10.0, p=0.2)
    og = O.OGridData(R, dense.astype(np.float64), active, background=-10.0)
    # the oracle's grid must allocate exactly the library's leaves
    mn, mx = np.array([-1.5, -1.3, -1.6], np.float32), np.array([1.5, 1.4, 1.2], np.float32)
    shape = (23, 31, 17) if mode == 0 else R
    rng = np.random.default_rng(9)
    old = rng.random((19, 22, 25)) < 0.7
    init = rng.random(shape) < 0.8
    mask = torch.from_numpy(init.astype(np.uint8)).cuda()
    oldt = torch.from_numpy(old.astype(np.uint8)).cuda()
    L.call("pvdb_occupancy", g.handle, mode, L.ptr(mask), L.i32arr(list(shape)),
           L.f32arr(mn), L.f32arr(mx), -4.6, 0.5, 1e-3, L.ptr(oldt) if mode == 1 else None,
           L.i32arr(list(old.shape)), None)
    ref, margin = OL.occupancy(mode, og, shape, mn, mx, -4.6, 0.5, 1e-3, mask=init,
                               old_mask=old if mode == 1 else None)
    _assert_mask(mask.cpu().numpy().astype(bool), margin, ref, 1e-3)
    assert ref.any() and not ref.all()


def test_near_cams_against_reference(lib, gold):
    from plenvdb_gb300 import lifecycle as LC
    R = gold["near_mask"].shape
    g, dense, active = _sparse(R, 10, bg=-10.0, p=0.5)
    mn, mx = gold["near_box"]
    LC.maskout_near_cam_vox(g, gold["near_cams"], float(gold["near_clip"]), mn, mx)
    got = g.get_dense_grid().reshape(R)
    # setValuesOn_bymask touches active voxels only
    ref = np.where(gold["near_mask"] & (active > 0), np.float32(-100), dense)
    np.testing.assert_array_equal(got, ref)
    assert (gold["near_mask"] & (active > 0)).any()


def test_count_views_against_reference(lib, gold):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    ro, rd = gold["cv_ro"], gold["cv_rd"]
    mn, mx = gold["cv_box"]
    voxel_size, near, stepsize = (float(v) for v in gold["cv_params"])
    reso = tuple(int(r) for r in gold["cv_reso"])
    cnt = LC.voxel_count_views(torch.from_numpy(ro), torch.from_numpy(rd), [1] * ro.shape[0],
                               near, 6.0, stepsize, reso, voxel_size, mn, mx)
    n_samples = int(np.linalg.norm(np.array(reso) + 1) / stepsize) + 1
    stepdist = float(np.float32(stepsize) * np.float32(voxel_size))
    near1 = np.zeros(reso, bool)
    for v in range(ro.shape[0]):
        s = OL.view_weight_sums(ro[v], rd[v], reso, mn, mx, near, stepdist, n_samples)
        near1 |= np.abs(s - 1) < 1e-4
    got = cnt.cpu().numpy()[0, 0]
    ref = gold["cv_count"][0, 0]
    assert not ((got != ref) & ~near1).any()
    assert got.max() >= 2


def test_count_views_larger_against_oracle(lib):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    from plenvdb_gb300.scene import CameraConfig, random_rays
    reso = (40, 36, 44)
    mn, mx = [-1.5] * 3, [1.5] * 3
    ro, rd, _ = random_rays(CameraConfig(), 6000, 3, seed=12)
    ro, rd = ro.reshape(3, 2000, 3), rd.reshape(3, 2000, 3)
    cnt = LC.voxel_count_views(torch.from_numpy(ro), torch.from_numpy(rd), [1] * 3, 2.0, 6.0,
                               0.5, reso, 3.0 / 40, mn, mx, irregular_shape=True)
    n_samples = int(np.linalg.norm(np.array(reso) + 1) / 0.5) + 1
    stepdist = float(np.float32(0.5) * np.float32(3.0 / 40))
    ref = np.zeros(reso)
    near1 = np.zeros(reso, bool)
    for v in range(3):
        s = OL.view_weight_sums(ro[v], rd[v], reso, mn, mx, 2.0, stepdist, n_samples)
        ref += s > 1
        near1 |= np.abs(s - 1) < 1e-4
    got = cnt.cpu().numpy()[0, 0]
    assert not ((got != ref) & ~near1).any()
    assert ref.max() == 3 and (ref == 0).any()


# ------------------------------------------------------------------ rays
def test_rays_against_reference(lib, gold):
    import torch
    from plenvdb_gb300 import rays as RY
    H, W = (int(v) for v in gold["rays_HW"])
    for n in range(int(gold["rays_ncases"])):
        mode, inv, fx, fy, ndc, seed = (int(v) for v in gold[f"rays{n}_flags"])
        mode = ["center", "lefttop", "random"][mode]
        torch.manual_seed(seed)
        o, d, v = RY.get_rays_of_a_view(H, W, gold["rays_K"], torch.from_numpy(gold["rays_c2w"]),
                                        bool(ndc), bool(inv), bool(fx), bool(fy), mode=mode)
        np.testing.assert_array_equal(o.cpu().numpy(), gold[f"rays{n}_o"], err_msg=str(n))
        np.testing.assert_array_equal(d.cpu().numpy(), gold[f"rays{n}_d"], err_msg=str(n))
        np.testing.assert_array_equal(v.cpu().numpy(), gold[f"rays{n}_v"], err_msg=str(n))


def test_hit_coarse_geo_and_maskcache_sampling(lib):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    from plenvdb_gb300 import rays as RY
    from plenvdb_gb300.scene import SceneConfig, scene_mask, sphere_poses
    R = 48
    mask = scene_mask(SceneConfig(reso=R, n_ellipsoids=5, seed=3)).astype(bool)
    mn, mx = [-1.5] * 3, [1.5] * 3
    mc = LC.MaskGrid(mask=torch.from_numpy(mask).cuda(), xyz_min=mn, xyz_max=mx)
    H, W = 60, 50
    K = np.array([[70.0, 0, 25.0], [0, 70.0, 30.0], [0, 0, 1]])
    poses = sphere_poses(3, 4.03, seed=2)
    voxel_size = 3.0 / R
    model = type("M", (), {"xyz_min": mn, "xyz_max": mx, "voxel_size": voxel_size,
                           "mask_cache": mc})()
    rng = np.random.default_rng(4)
    imgs = [rng.random((H, W, 3)).astype(np.float32) for _ in poses]
    out = RY.get_training_rays_in_maskcache_sampling(
        imgs, [torch.from_numpy(p) for p in poses], [(H, W)] * 3, [K] * 3, False, False, False,
        False, model, {"near": 2.0, "stepsize": 0.5})
    rgb_tr, ro_tr, rd_tr, vd_tr, imsz = out
    stepdist = float(np.float32(0.5) * np.float32(voxel_size))
    top = 0
    for p, img, n in zip(poses, imgs, imsz):
        o, d, v = OL.get_rays(H, W, K, p, False, False, False)
        hit = OL.hit_coarse_geo(o, d, mn, mx, 2.0, stepdist, mask).reshape(H, W)
        assert n == int(hit.sum()) and 0 < n < H * W
        np.testing.assert_array_equal(ro_tr[top:top + n].cpu().numpy(), o[hit])
        np.testing.assert_array_equal(rd_tr[top:top + n].cpu().numpy(), d[hit])
        np.testing.assert_array_equal(vd_tr[top:top + n].cpu().numpy(), v[hit])
        np.testing.assert_array_equal(rgb_tr[top:top + n].cpu().numpy(), img[hit])
        top += n
    assert rgb_tr.shape[0] == top


# ------------------------------------------------------ files and resume
def test_merged_files_round_trip_into_renderer(lib, tmp_path):
    import torch
    from plenvdb_gb300 import lifecycle as LC
    from plenvdb_gb300.renderer import MGRenderer
    from plenvdb_gb300.scene import SceneConfig, build_grids, rgbnet_init, scene_mask, sphere_poses
    scfg = SceneConfig(reso=40, n_ellipsoids=4, seed=5)
    dg, kg = build_grids(scfg)
    mask = torch.from_numpy(scene_mask(scfg)).cuda()
    merged = LC.merge_compress(dg, kg, mask)
    LC.save_merged(str(tmp_path), merged)
    den, col, index, N = LC.load_merged(str(tmp_path))
    assert N == merged["N"]
    np.testing.assert_array_equal(index, merged["index"].cpu().numpy())
    net = [t.numpy() for t in rgbnet_init(seed=1)]
    params = [net[0].T.copy(), net[1], net[2].T.copy(), net[3], net[4].T.copy(), net[5]]
    K = np.array([[60.0, 0, 20], [0, 60.0, 20], [0, 0, 1]], np.float32)
    imgs = []
    for idx in (index, str(tmp_path / "mergedidxs.npz")):
        r = MGRenderer(12, 27, 128, 3)
        r.load_data(den, col, idx, N)
        r.load_params(*params)
        r.setScene([40] * 3, K, scfg.xyz_min, scfg.xyz_max)
        r.setKwargs(2.0, 6.0, 0.5 * 3.0 / 40, -4.6, 0.5, 1e-4, 1.0, False, 40, 40)
        r.input_a_c2w(sphere_poses(1, 4.03, seed=1)[0])
        r.render_an_image()
        imgs.append(r.output_an_image())
    np.testing.assert_array_equal(imgs[0], imgs[1])
    assert imgs[0].std() > 0


def test_checkpoint_resume_is_bitwise(lib, tmp_path):
    import torch
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays, rgbnet_init
    from plenvdb_gb300.trainer import FineStageConfig, FineStageTrainer
    scfg = SceneConfig(reso=48, n_ellipsoids=5, seed=7)
    cfg = FineStageConfig(reso=48, precision=1)
    ro, rd, vd = random_rays(CameraConfig(), 4 * 2048, 5, seed=3)
    tgt = np.random.default_rng(1).random((ro.shape[0], 3)).astype(np.float32)
    batches = [tuple(torch.from_numpy(a[b * 2048:(b + 1) * 2048]).cuda() for a in (ro, rd, vd, tgt))
               for b in range(4)]

    def trainer():
        dg, kg = build_grids(scfg)
        return FineStageTrainer(dg, kg, rgbnet_init(seed=2), cfg, max_rays=2048)

    a = trainer()
    for i in range(3):
        a.step(*batches[i % 4])
    a.save_checkpoint(str(tmp_path / "fine"), global_step=3)
    la = [float(a.step(*batches[i % 4])) for i in range(3, 7)]
    b = trainer()
    assert b.load_checkpoint(str(tmp_path / "fine")) == 3
    lb = [float(b.step(*batches[i % 4])) for i in range(3, 7)]
    torch.cuda.synchronize()
    assert la == lb
    np.testing.assert_array_equal(a.density.get_dense_grid(), b.density.get_dense_grid())
    np.testing.assert_array_equal(a.k0.get_dense_grid(), b.k0.get_dense_grid())
    assert torch.equal(a.params, b.params) and torch.equal(a.exp_avg_sq, b.exp_avg_sq)
    # the mask cache of the saved checkpoint, as MaskGrid(path=...) builds it
    from plenvdb_gb300 import lifecycle as LC
    mg = LC.MaskGrid(path=str(tmp_path / "fine_last.npz"), mask_cache_thres=1e-3)
    assert mg.shape == (48, 48, 48) and 0 < int(mg.mask.sum()) < 48 ** 3


def test_merge_one_grid_only(lib):
    """Density-only and colour-only compression (the other rows not written)."""
    import torch
    from plenvdb_gb300 import lifecycle as LC
    R = (19, 23, 17)
    dg, dd, _ = _sparse(R, 11)
    kg, kd, _ = _sparse(R, 12, C=12, bg=0.0)
    mask = np.random.default_rng(13).random(R) < 0.3
    m = torch.from_numpy(mask).cuda()
    a = LC.merge_compress(dg, None, m, row_dtype="float32")
    b = LC.merge_compress(None, kg, m, row_dtype="float32")
    idx, den, col = OL.merge(dd, kd, mask, dtype=np.float32)
    assert a["col"] is None and b["den"] is None
    np.testing.assert_array_equal(a["index"].cpu().numpy(), idx)
    np.testing.assert_array_equal(b["index"].cpu().numpy(), idx)
    np.testing.assert_array_equal(a["den"].cpu().numpy(), den)
    np.testing.assert_array_equal(b["col"].cpu().numpy(), col)


def test_rescaled_mask_cache_without_old_cache(lib):
    """The rebuild after rescaling with no previous mask cache: only the pooled
    alpha decides (the old-cache lookup counts as all set)."""
    from plenvdb_gb300 import lifecycle as LC
    R = (21, 18, 26)
    g, dense, active = _sparse(R, 14, bg=-10.0, p=0.25)
    og = O.OGridData(R, dense.astype(np.float64), active, background=-10.0)
    mn, mx = [-1.5] * 3, [1.5] * 3
    new = LC.rescaled_mask_cache(None, g, mn, mx, -4.6, 0.5, 1e-3)
    ref, margin = OL.occupancy(1, og, R, mn, mx, -4.6, 0.5, 1e-3)
    _assert_mask(new.mask.cpu().numpy().astype(bool), margin, ref, 1e-3)
    assert ref.any() and not ref.all()
