"""GPU parity of the leaf store (lookup, trilinear forward/backward, voxel Adam,
TV, dense copies, save/load) against the reference's NanoVDB golden vectors
and the CPU oracle."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _fill_leaves(vdb, padded_values):
    """Write every in-leaf voxel value (active or not) from a padded dense array."""
    import torch
    data, _, _, _, origin = vdb.device_views()
    org = origin.cpu().numpy()
    v = np.arange(512)
    off = np.stack([v >> 6, (v >> 3) & 7, v & 7], -1)
    coords = org[:, None, :] + off[None]
    pv = np.asarray(padded_values, np.float32)
    if pv.ndim == 3:
        pv = pv[..., None]
    vals = pv[coords[..., 0], coords[..., 1], coords[..., 2]]
    data.copy_(torch.from_numpy(np.ascontiguousarray(vals)).cuda())
    torch.cuda.synchronize()


@pytest.fixture(scope="module")
def golden_grids(golden, lib):
    from plenvdb_gb300 import ColorVDB, DensityVDB
    R = [int(r) for r in golden["reso"]]
    dg = DensityVDB.from_mask(R, golden["active"], background=float(golden["background"]))
    kg = ColorVDB.from_mask(R, golden["active"], background=0.0, n=12)
    _fill_leaves(dg, golden["density"])
    _fill_leaves(kg, golden["k0"])
    return dg, kg


def test_topology_matches_nanovdb(golden, golden_grids):
    dg, _ = golden_grids
    _, ch, nleaf, nact, bg = dg.info()
    assert nleaf == int(golden["alloc"].sum())
    assert nact == int(golden["active"].sum())
    assert ch == 1 and bg == float(golden["background"])


def test_lookup_bit_exact(golden, golden_grids):
    dg, _ = golden_grids
    ijk = golden["lookup_ijk"]
    val, act = dg.forward_single(ijk[:, 0], ijk[:, 1], ijk[:, 2], with_active=True)
    np.testing.assert_array_equal(val, golden["lookup_val"])
    np.testing.assert_array_equal(act.astype(np.uint8), golden["lookup_active"])


def test_density_forward_bit_exact(golden, golden_grids):
    dg, _ = golden_grids
    xyz = golden["fwd_xyz"]
    out = dg.forward(xyz[:, 0], xyz[:, 1], xyz[:, 2])
    np.testing.assert_array_equal(out, golden["fwd_density"])


def test_color_forward_bit_exact(golden, golden_grids):
    _, kg = golden_grids
    xyz = golden["fwd_xyz"]
    out = kg.forward(xyz[:, 0], xyz[:, 1], xyz[:, 2]).reshape(-1, 12)
    np.testing.assert_array_equal(out, golden["fwd_color"])


def test_forward_device_tensors(golden, golden_grids):
    import torch
    dg, kg = golden_grids
    xyz = torch.from_numpy(golden["fwd_xyz"]).cuda()
    out = dg.forward(xyz[:, 0].contiguous(), xyz[:, 1].contiguous(), xyz[:, 2].contiguous())
    assert out.is_cuda
    np.testing.assert_array_equal(out.cpu().numpy(), golden["fwd_density"])


@pytest.mark.parametrize("kind", ["density", "color"])
def test_backward_matches_reference_and_is_deterministic(golden, golden_grids, kind):
    dg, kg = golden_grids
    g = dg if kind == "density" else kg
    xyz = golden["bwd_xyz"]
    grad = golden["bwd_gdens"] if kind == "density" else golden["bwd_gcol"]
    from plenvdb_gb300 import _lib as L
    outs = []
    for _ in range(2):
        _fill_leaves_grad_zero(g)
        g.backward(xyz[:, 0], xyz[:, 1], xyz[:, 2], grad.reshape(-1))
        outs.append(g.get_dense_grid(which=L.WHICH_GRAD))
    assert np.array_equal(outs[0], outs[1]), "backward is not bitwise reproducible"
    ref = golden["bwd_density"] if kind == "density" else golden["bwd_color"]
    np.testing.assert_allclose(outs[0].reshape(ref.shape), ref, rtol=1e-5, atol=2e-6)


def _fill_leaves_grad_zero(g):
    import torch
    _, grad, _, _, _ = g.device_views()
    grad.zero_()
    torch.cuda.synchronize()


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("kind", ["d", "c"])
def test_voxel_adam_matches_reference(golden, lib, mode, kind):
    import torch
    from plenvdb_gb300 import ColorOpt, ColorVDB, DensityOpt, DensityVDB
    R = [int(r) for r in golden["reso"]]
    stepsz, eps, b0, b1 = (float(x) for x in golden["adam_hyper"])
    act = golden["active"]
    if kind == "d":
        g = DensityVDB.from_mask(R, act, background=float(golden["background"]))
        _fill_leaves(g, golden["density"])
        opt = DensityOpt(g, 1.0, eps, b0, b1)
        grad, m, v = golden["adam_grad_d"], golden["adam_m_d"], golden["adam_v_d"]
    else:
        g = ColorVDB.from_mask(R, act, background=0.0, n=12)
        _fill_leaves(g, golden["k0"])
        opt = ColorOpt(g, 1.0, eps, b0, b1)
        grad, m, v = golden["adam_grad_c"], golden["adam_m_c"], golden["adam_v_c"]
    # lr such that the host step size equals the fixture's (step 1: sqrt(1-b1)/(1-b0))
    lr = np.float32(stepsz) / (np.float32(np.sqrt(np.float32(1) - np.float32(b1))) /
                               (np.float32(1) - np.float32(b0)))
    opt.setLr(float(lr))
    g.copyFromDense(grad.reshape(-1), which=1)
    ma, mb = opt._moments()
    for h, arr in ((ma, m), (mb, v)):
        L = __import__("plenvdb_gb300._lib", fromlist=["x"])
        a = np.ascontiguousarray(arr.reshape(-1).astype(np.float32))
        L.call("pvdb_grid_copy_from_dense", h, 0, L.ptr(a), a.size, L.MEM_HOST, None)
    if mode == 2:
        opt.set_pervoxel_lr(golden["adam_lr"].reshape(-1))
    opt.step(mode)
    out = g.get_dense_grid().reshape(golden[f"adam_{kind}{mode}_data"].shape)
    np.testing.assert_allclose(out, golden[f"adam_{kind}{mode}_data"], rtol=3e-6, atol=2e-6)


def test_tv_matches_oracle(lib):
    import torch
    from plenvdb_gb300 import ColorVDB
    rng = np.random.default_rng(5)
    R = 19
    act = (rng.random((R, R, R)) < 0.5).astype(np.uint8)
    vals = rng.normal(0, 1, (R, R, R, 3)).astype(np.float32)
    g = ColorVDB.from_mask([R] * 3, act, background=-1.0, n=3)
    g.copyFromDense(vals.reshape(-1))
    grad0 = rng.normal(0, 1, (R, R, R, 3)).astype(np.float32)
    grad0[rng.random(grad0.shape) < 0.5] = 0
    og = O.OGridData((R,) * 3, np.where(act[..., None] > 0, vals, -1.0), act, background=-1.0)
    for dense_mode in (0, 1):
        g.copyFromDense(grad0.reshape(-1), which=1)
        g.total_variation_add_grad(0.6, 1.2, 1.8, dense_mode)
        got = g.get_dense_grid(which=1).reshape(R, R, R, 3)
        gp = O.OGridData((R,) * 3, grad0, act, background=0.0).p_values.copy()
        O.tv(og, gp, 0.1, 0.2, 0.3, dense_mode)
        want = og.unpad(gp)
        want = np.where(act[..., None] > 0, want, grad0 * 0)  # inactive voxels keep 0 grad
        np.testing.assert_allclose(got * (act[..., None] > 0), want * (act[..., None] > 0),
                                   rtol=1e-5, atol=1e-6)


def test_dense_roundtrip_and_mask(lib):
    from plenvdb_gb300 import DensityVDB
    rng = np.random.default_rng(1)
    R = [13, 17, 9]
    g = DensityVDB(R, 1)
    a = rng.normal(size=R).astype(np.float32)
    g.copyFromDense(a.reshape(-1))
    np.testing.assert_array_equal(g.get_dense_grid().reshape(R), a)
    mask = rng.random(R) < 0.3
    g.setValuesOn_bymask(mask.reshape(-1), -100.0)
    b = g.get_dense_grid().reshape(R)
    np.testing.assert_array_equal(b[mask], -100.0)
    np.testing.assert_array_equal(b[~mask], a[~mask])


def test_save_load_and_corruption(tmp_path, lib):
    from plenvdb_gb300 import ColorVDB
    from plenvdb_gb300 import _lib as L
    rng = np.random.default_rng(2)
    R = [16, 16, 16]
    act = (rng.random(R) < 0.2).astype(np.uint8)
    g = ColorVDB.from_mask(R, act, background=0.0, n=6)
    g.copyFromDense(rng.normal(size=R + [6]).astype(np.float32).reshape(-1))
    p = str(tmp_path / "color.vdb")
    g.save_to(p)
    h = ColorVDB(R, 6)
    h.load_from(p)
    np.testing.assert_array_equal(h.get_dense_grid(), g.get_dense_grid())
    assert h.info()[2:4] == g.info()[2:4]
    raw = bytearray(open(p, "rb").read())
    raw[100] ^= 0xFF
    open(p, "wb").write(bytes(raw))
    with pytest.raises(L.PvdbError) as e:
        h.load_from(p)
    assert e.value.code == L.PVDB_ERR_IO
    with pytest.raises(L.PvdbError):
        h.load_from(str(tmp_path / "missing.vdb"))


def test_injected_allocation_failure(lib):
    from plenvdb_gb300 import DensityVDB
    from plenvdb_gb300 import _lib as L
    L.load().pvdb_debug_fail_next_allocs(1)
    with pytest.raises(L.PvdbError) as e:
        DensityVDB([8, 8, 8], 1)
    assert e.value.code == L.PVDB_ERR_NOMEM
    g = DensityVDB([8, 8, 8], 1)  # the library stays usable
    assert g.info()[2] == 1
