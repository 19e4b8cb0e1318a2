"""Pins the lifecycle oracle (oracle/lifecycle.py) to the reference's own
Python code, run by tests/golden/make_lifecycle_golden.py: rays, batch
indices, merged compression, rescaling, the three mask-cache builds,
near-camera masking and the per-view voxel counts. CPU only."""
import os

import numpy as np
import pytest
import torch

from oracle import lifecycle as OL
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "lifecycle_golden.npz"))


def test_rays_match_reference(gold):
    H, W = (int(v) for v in gold["rays_HW"])
    K, c2w = gold["rays_K"], gold["rays_c2w"]
    for n in range(int(gold["rays_ncases"])):
        mode, inv, fx, fy, ndc, seed = (int(v) for v in gold[f"rays{n}_flags"])
        mode = ["center", "lefttop", "random"][mode]
        jitter = None
        if mode == "random":
            torch.manual_seed(seed)
            jitter = (torch.rand(H, W).numpy(), torch.rand(H, W).numpy())
        o, d, v = OL.get_rays(H, W, K, c2w, inv, fx, fy, mode, jitter, ndc=bool(ndc))
        np.testing.assert_array_equal(o, gold[f"rays{n}_o"], err_msg=str(n))
        np.testing.assert_array_equal(d, gold[f"rays{n}_d"], err_msg=str(n))
        np.testing.assert_array_equal(v, gold[f"rays{n}_v"], err_msg=str(n))


def test_batch_indices_match_reference(gold):
    from plenvdb_gb300.rays import batch_indices_generator
    np.random.seed(7)
    g = batch_indices_generator(50, 16)
    got = np.stack([next(g).numpy() for _ in range(8)])
    np.testing.assert_array_equal(got, gold["batches"])


def test_merge_matches_reference(gold):
    idx, den, col = OL.merge(gold["merge_den"], gold["merge_col"], gold["merge_mask"])
    np.testing.assert_array_equal(idx, gold["merge_idxs"].astype(np.int32))
    assert den.dtype == np.float16 and col.dtype == np.float16
    np.testing.assert_array_equal(den.view(np.uint16), gold["merge_den_rows"].view(np.uint16))
    np.testing.assert_array_equal(col.view(np.uint16), gold["merge_col_rows"].view(np.uint16))
    assert np.isinf(col.astype(np.float32)).any()  # the FP16 overflow case is covered


def test_resample_matches_reference(gold):
    for n in range(2):
        out = OL.resample(gold[f"scale{n}_src"], gold[f"scale{n}_dst"])
        ref = gold[f"scale{n}_out"]
        np.testing.assert_array_equal(out, ref)


def _occ_setup(gold):
    dens = gold["occ_dens"]
    g = O.OGridData(dens.shape, dens.astype(np.float64), np.ones(dens.shape, np.uint8),
                    background=0.0)
    mn, mx = gold["occ_box"]
    shift, interval, thres = (float(v) for v in gold["occ_params"])
    return g, mn, mx, shift, interval, thres


def _assert_mask(got, margin, ref, thres):
    diff = got != ref
    near = np.abs(margin.astype(np.float64) - thres) <= 1e-5 * max(thres, 1e-30)
    assert not (diff & ~near).any(), f"{int((diff & ~near).sum())} voxels differ"
    assert ref.any() and not ref.all()


def test_occupancy_update_matches_reference(gold):
    g, mn, mx, shift, interval, thres = _occ_setup(gold)
    old = gold["occ_old"]
    got, margin = OL.occupancy(0, g, old.shape, mn, mx, shift, interval, thres, mask=old)
    _assert_mask(got, margin, gold["occ_mode0"], thres)


def test_occupancy_rescale_rebuild_matches_reference(gold):
    g, mn, mx, shift, interval, thres = _occ_setup(gold)
    got, margin = OL.occupancy(1, g, g.reso, mn, mx, shift, interval, thres,
                               old_mask=gold["occ_old"])
    _assert_mask(got, margin, gold["occ_mode1"], thres)


def test_occupancy_from_checkpoint_matches_reference(gold):
    g, mn, mx, shift, interval, thres = _occ_setup(gold)
    got, margin = OL.occupancy(2, g, g.reso, mn, mx, shift, interval, thres)
    _assert_mask(got, margin, gold["occ_mode2"], thres)


def test_near_cameras_match_reference(gold):
    mn, mx = gold["near_box"]
    got = OL.near_cam_mask(gold["near_mask"].shape, gold["near_cams"], float(gold["near_clip"]),
                           mn, mx)
    np.testing.assert_array_equal(got, gold["near_mask"])
    assert got.any() and not got.all()


def test_view_counts_match_reference(gold):
    ro, rd = gold["cv_ro"], gold["cv_rd"]
    mn, mx = gold["cv_box"]
    voxel_size, near, stepsize = (float(v) for v in gold["cv_params"])
    reso = tuple(int(r) for r in gold["cv_reso"])
    n_samples = int(np.linalg.norm(np.array(reso) + 1) / stepsize) + 1
    stepdist = float(np.float32(stepsize) * np.float32(voxel_size))
    count = np.zeros(reso)
    near1 = np.zeros(reso, bool)
    for v in range(ro.shape[0]):
        s = OL.view_weight_sums(ro[v], rd[v], reso, mn, mx, near, stepdist, n_samples)
        count += s > 1
        near1 |= np.abs(s - 1) < 1e-4
    ref = gold["cv_count"][0, 0]
    diff = count != ref
    assert not (diff & ~near1).any(), f"{int((diff & ~near1).sum())} voxels differ"
    assert ref.max() >= 2 and (ref == 0).any()
