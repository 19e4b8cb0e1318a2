"""Pins the CPU oracle to the reference's own NanoVDB (golden vectors produced
by tests/golden/make_golden.py through oracle/ref_harness.cpp)."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def grids(golden):
    R = tuple(int(r) for r in golden["reso"])
    bg = float(golden["background"])
    gd = O.OGridData(R, golden["density"], golden["active"], background=bg, alloc=golden["alloc"])
    gk = O.OGridData(R, golden["k0"], golden["active"], background=0.0, alloc=golden["alloc"])
    return gd, gk


def test_lookup_bit_exact(golden, grids):
    """ReadAccessor::getValue/isActive: stored value in allocated leaves (active
    or not), background outside, including negative / beyond-padding coords."""
    gd, _ = grids
    val, act = O.lookup(gd, golden["lookup_ijk"])
    np.testing.assert_array_equal(val[:, 0].astype(np.float32), golden["lookup_val"])
    np.testing.assert_array_equal(act, golden["lookup_active"])


def test_density_forward_bit_exact(golden, grids):
    gd, _ = grids
    out = O.sample(gd, golden["fwd_xyz"], fp32=True)[:, 0].astype(np.float32)
    np.testing.assert_array_equal(out, golden["fwd_density"])
    # fp64 truth within float rounding
    out64 = O.sample(gd, golden["fwd_xyz"])[:, 0]
    np.testing.assert_allclose(out64, golden["fwd_density"], rtol=1e-5, atol=1e-5)


def test_color_forward_bit_exact(golden, grids):
    _, gk = grids
    out = O.sample(gk, golden["fwd_xyz"], fp32=True).astype(np.float32)
    np.testing.assert_array_equal(out, golden["fwd_color"])


def test_density_backward(golden, grids):
    gd, _ = grids
    g = O.sample_backward(gd, golden["bwd_xyz"], golden["bwd_gdens"].astype(np.float64))[..., 0]
    # the reference adds float contributions (here sequentially); the oracle sums in double
    np.testing.assert_allclose(g, golden["bwd_density"], rtol=1e-5, atol=2e-6)
    # corners outside allocated leaves are dropped: those voxels stay zero
    alloc_vox = np.repeat(np.repeat(np.repeat(golden["alloc"], 8, 0), 8, 1), 8, 2)[:20, :20, :20]
    assert np.all(golden["bwd_density"][alloc_vox == 0] == 0)


def test_color_backward(golden, grids):
    _, gk = grids
    g = O.sample_backward(gk, golden["bwd_xyz"], golden["bwd_gcol"].astype(np.float64))
    np.testing.assert_allclose(g, golden["bwd_color"], rtol=1e-5, atol=2e-6)


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("kind", ["d", "c"])
def test_voxel_adam(golden, mode, kind):
    R = tuple(int(r) for r in golden["reso"])
    stepsz, eps, b0, b1 = (float(x) for x in golden["adam_hyper"])
    if kind == "d":
        data, grad, m, v = golden["density"], golden["adam_grad_d"], golden["adam_m_d"], golden["adam_v_d"]
        bg = float(golden["background"])
    else:
        data, grad, m, v = golden["k0"], golden["adam_grad_c"], golden["adam_m_c"], golden["adam_v_c"]
        bg = 0.0
    g = O.OGridData(R, data, golden["active"], background=bg, alloc=golden["alloc"])
    pad = lambda a: O.OGridData(R, a, golden["active"], background=0.0,  # noqa: E731
                                alloc=golden["alloc"]).p_values.copy()
    gp, mp, vp = pad(grad), pad(m), pad(v)
    lrp = O.OGridData(R, golden["adam_lr"], golden["active"], alloc=golden["alloc"]).p_values.copy()
    out = O.adam(g, gp, mp, vp, lrp, stepsz, eps, b0, b1, mode, fp32=True)
    mg = O.OGridData(R, np.zeros_like(np.asarray(m)), golden["active"], background=0.0,
                     alloc=golden["alloc"])

    def dense(a):  # moments read through the leaf rules (background 0 outside leaves)
        d = mg.dense(a)
        return d[..., 0] if kind == "d" else d
    ref = golden[f"adam_{kind}{mode}_data"]
    # inside allocated leaves compare values; outside they read the background
    got = g.dense(out)
    got = got[..., 0] if kind == "d" else got
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-6)
    np.testing.assert_allclose(dense(mp), golden[f"adam_{kind}{mode}_m"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(dense(vp), golden[f"adam_{kind}{mode}_v"], rtol=1e-6, atol=1e-9)
    # voxels that are inactive keep their value
    act = golden["active"].astype(bool)
    base = g.dense()
    base = base[..., 0] if kind == "d" else base
    assert np.array_equal(got[~act], base[~act])


def test_index_density_matches_nanovdb(golden):
    """The render march's index-grid lookups (renderer.cu:253, 271-300) against
    the reference's NanoVDB accessor: isActive(Round(xyz)) exactly (rint ties
    included), the trilinear density within float rounding (the golden vectors
    use the count pass's association, the oracle the fill pass's)."""
    rows = golden["idx_rows"].astype(np.int32)
    out32, act = O.index_density(rows, golden["idx_den_rows"], golden["idx_xyz"], fp32=True)
    np.testing.assert_array_equal(act, golden["idx_active_round"].astype(bool))
    np.testing.assert_allclose(out32, golden["idx_density"], rtol=1e-5, atol=2e-6)
    out64, _ = O.index_density(rows, golden["idx_den_rows"], golden["idx_xyz"], fp32=False)
    np.testing.assert_allclose(out64, golden["idx_density"], rtol=1e-5, atol=2e-6)


def test_render_oracle_fp32_tracks_fp64(golden):
    """Render march restatement: the float-mirroring mode stays within float
    rounding of FP64, and a pixel without a colour sample is the background."""
    from plenvdb_gb300.scene import rgbnet_init, sphere_poses
    rows = golden["idx_rows"].astype(np.int32)
    R = rows.shape[0]
    den = golden["idx_den_rows"] + np.float32(3.0)
    rng = np.random.default_rng(0)
    col = rng.normal(0, 0.1, (den.shape[0], 12)).astype(np.float32)
    col[0] = 0.0
    net = [t.numpy().astype(np.float64) for t in rgbnet_init(seed=1)]
    mlp = O.MLPWeights(*net, c0=12, pe=4)
    K = np.array([[60.0, 0, 24], [0, 60.0, 24], [0, 0, 1]], np.float32)
    pose = sphere_poses(1, 4.03, seed=2)[0]
    kw = dict(near=2.0, stepdist=0.5 * 3.0 / R, act_shift=-4.6, interval=0.5, thres=1e-4,
              bg=1.0, t_stop=1e-4)
    lo, hi = [-1.5] * 3, [1.5] * 3
    r32, n32, _ = O.render_pixels(rows, den, col, mlp, K, pose, lo, hi, 48, 48, fp32=True, **kw)
    r64, n64, _ = O.render_pixels(rows, den, col, mlp, K, pose, lo, hi, 48, 48, fp32=False, **kw)
    assert (n64 > 0).mean() > 0.1
    same = n32 == n64
    assert same.mean() > 0.99
    np.testing.assert_allclose(r32[same], r64[same], rtol=1e-5, atol=1e-6)
    assert np.all(r64[n64 == 0] == 1.0)
