"""The CUDA primitives of the DirectVoxGO path against golden vectors from the
reference's own torch-extension kernels run on a GB300
(tests/golden/dvgo_ext_golden.npz; render_utils_kernel.cu,
total_variation_kernel.cu, adam_upd_kernel.cu), through the C ABI.

Bit-exact: ray sampling, the mask cache, raw2alpha's forward, TV and dense
Adam. alpha2weight keeps the transmittance product in one FP32 fma where the
reference rounds a double product to float: equal but for double-rounding
ties (a few ulps at most). The two backward formulas form in FP32 what the
reference forms in double: within the stated ulps / relative bounds."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def G(lib):
    return np.load(os.path.join(ROOT, "tests", "golden", "dvgo_ext_golden.npz"))


def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def _cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_sample_pts_on_rays_matches_reference(G):
    import torch
    from plenvdb_gb300 import render_utils as RU
    near, far, step = (float(x) for x in G["sp_params"])
    out = RU.sample_pts_on_rays(_cuda(G["sp_rays_o"]), _cuda(G["sp_rays_d"]),
                                torch.from_numpy(G["sp_xyz_min"]), torch.from_numpy(G["sp_xyz_max"]),
                                near, far, step)
    pts, ob, rid, sid, ns, tmin, tmax = (x.cpu().numpy() for x in out)
    np.testing.assert_array_equal(tmin, G["sp_t_min"])
    np.testing.assert_array_equal(tmax, G["sp_t_max"])
    np.testing.assert_array_equal(ns, G["sp_n_steps"])
    np.testing.assert_array_equal(rid, G["sp_ray_id"])
    np.testing.assert_array_equal(sid, G["sp_step_id"])
    np.testing.assert_array_equal(ob, G["sp_mask_outbbox"].astype(bool))
    np.testing.assert_array_equal(pts, G["sp_pts"])


def test_maskcache_lookup_matches_reference(G):
    import torch
    from plenvdb_gb300 import render_utils as RU
    shape = tuple(int(s) for s in G["mc_shape"])
    world = np.unpackbits(G["mc_world"])[:int(np.prod(shape))].reshape(shape).astype(bool)
    out = RU.maskcache_lookup(_cuda(world), _cuda(G["mc_xyz"]), torch.from_numpy(G["mc_scale"]),
                              torch.from_numpy(G["mc_shift"]))
    np.testing.assert_array_equal(out.cpu().numpy(), G["mc_out"].astype(bool))


@pytest.mark.parametrize("tag,interval", [("05", 0.5), ("10", 1.0)])
def test_raw2alpha_matches_reference(G, tag, interval):
    from plenvdb_gb300 import render_utils as RU
    e, a = RU.raw2alpha(_cuda(G["ra_density"]), float(G["ra_params"][0]), interval)
    np.testing.assert_array_equal(e.cpu().numpy(), G[f"ra{tag}_exp"])
    np.testing.assert_array_equal(a.cpu().numpy(), G[f"ra{tag}_alpha"])
    # backward from the reference's exp: three FP32 products vs one double product
    g = RU.raw2alpha_backward(_cuda(G[f"ra{tag}_exp"]), _cuda(G[f"ra{tag}_grad_back"]), interval)
    g = g.cpu().numpy()
    rg = G[f"ra{tag}_grad"]
    assert np.array_equal(np.sign(g), np.sign(rg))
    assert _ulps(np.abs(g), np.abs(rg)).max() <= 3


def test_alpha2weight_matches_reference(G):
    from plenvdb_gb300 import render_utils as RU
    n_rays = int(G["aw_n_rays"])
    w, T, last, i_s, i_e = RU.alpha2weight(_cuda(G["aw_alpha"]),
                                           _cuda(G["aw_ray_id"].astype(np.int64)), n_rays)
    np.testing.assert_array_equal(i_s.cpu().numpy(), G["aw_i_start"])
    np.testing.assert_array_equal(i_e.cpu().numpy(), G["aw_i_end"])
    for got, want in ((T, G["aw_T"]), (w, G["aw_weight"]), (last, G["aw_last"])):
        d = _ulps(got.cpu().numpy(), want)
        assert d.max() <= 4 and (d == 0).mean() > 0.999
    # backward on the reference's own forward outputs
    g = RU.alpha2weight_backward(_cuda(G["aw_alpha"]), _cuda(G["aw_weight"]), _cuda(G["aw_T"]),
                                 _cuda(G["aw_last"]), _cuda(G["aw_i_start"]),
                                 _cuda(G["aw_i_end"]), n_rays, _cuda(G["aw_grad_weights"]),
                                 _cuda(G["aw_grad_last"]))
    g = g.cpu().numpy()
    rg = G["aw_grad"]
    np.testing.assert_allclose(g, rg, rtol=1e-5, atol=1e-6 * np.abs(rg).max())


@pytest.mark.parametrize("tag", ["c1d", "c1s", "c12s", "c12d"])
def test_tv_matches_reference(G, tag):
    from plenvdb_gb300 import ColorVDB, DensityVDB
    from plenvdb_gb300 import _lib as L
    p = G[f"tv{tag}_param"][0]  # [C, X, Y, Z]
    C_, X, Y, Z = p.shape
    g = DensityVDB([X, Y, Z], 1) if C_ == 1 else ColorVDB([X, Y, Z], C_)
    g.copyFromDense(np.ascontiguousarray(np.moveaxis(p, 0, -1)).reshape(-1))
    g.copyFromDense(np.ascontiguousarray(np.moveaxis(G[f"tv{tag}_grad_in"][0], 0, -1)).reshape(-1),
                    which=L.WHICH_GRAD)
    wx, wy, wz = (float(x) for x in G[f"tv{tag}_w"])
    g.total_variation_add_grad(wx, wy, wz, bool(G[f"tv{tag}_dense"]))
    got = g.get_dense_grid(which=L.WHICH_GRAD).reshape(X, Y, Z, C_)
    np.testing.assert_array_equal(np.moveaxis(got, -1, 0), G[f"tv{tag}_grad_out"][0])


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_adam_dense_matches_reference(G, mode):
    import torch
    from plenvdb_gb300 import _lib as L
    lr, b1, b2, eps = (float(x) for x in G["adam_params"])
    p = _cuda(G[f"adam{mode}_p0"])
    m, v = torch.zeros_like(p), torch.zeros_like(p)
    perlr = _cuda(G[f"adam{mode}_perlr"]) if mode == 2 else None
    for step in (1, 2, 3):
        g = _cuda(G[f"adam{mode}_g{step}"])
        L.call("pvdb_adam_dense", L.ptr(p), L.ptr(g), L.ptr(m), L.ptr(v), L.ptr(perlr), p.numel(),
               step, b1, b2, lr, eps, mode, L.stream_of())
        torch.cuda.synchronize()
        np.testing.assert_array_equal(m.cpu().numpy(), G[f"adam{mode}_m{step}"])
        np.testing.assert_array_equal(v.cpu().numpy(), G[f"adam{mode}_v{step}"])
        np.testing.assert_array_equal(p.cpu().numpy(), G[f"adam{mode}_p{step}"])
