"""The oracle's restatement of the DirectVoxGO torch-extension math against
golden vectors from the reference's own kernels run on a GB300
(tests/golden/dvgo_ext_golden.npz, written by make_dvgo_ext_golden.py from
render_utils_kernel.cu, total_variation_kernel.cu and adam_upd_kernel.cu).

Bit-exact: ray sampling (t_min/t_max, N_steps, points, ray/step ids, the
out-of-bbox mask), the mask-cache lookup, alpha2weight and its backward, TV
and dense Adam in FP32 mode. raw2alpha goes through exp/pow, whose last bit
differs between CUDA's and the host's libm: within a few ulps."""
import os

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def G():
    return np.load(os.path.join(ROOT, "tests", "golden", "dvgo_ext_golden.npz"))


def _ulps(a, b):
    """Distance in float32 ulps (same-sign finite values)."""
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def _params(G):
    near, far, step = G["sp_params"]
    return O.march_params(G["sp_xyz_min"], G["sp_xyz_max"], float(near), float(step), -4.6, 0.5,
                          1e-4, far=float(far))


def test_ray_count_exact(G):
    tmin, tmax, ns = O.ray_count(G["sp_rays_o"], G["sp_rays_d"], _params(G))
    np.testing.assert_array_equal(tmin, G["sp_t_min"])
    np.testing.assert_array_equal(tmax, G["sp_t_max"])
    np.testing.assert_array_equal(ns, G["sp_n_steps"])
    # the fixture holds every ray kind: misses (1 sample), single and long rays
    assert (G["sp_n_steps"] == 1).sum() >= 10 and G["sp_n_steps"].max() > 300


def test_ray_points_exact(G):
    pts, ob, rid, sid = O.ray_points(G["sp_rays_o"], G["sp_rays_d"], _params(G))
    np.testing.assert_array_equal(rid, G["sp_ray_id"])
    np.testing.assert_array_equal(sid, G["sp_step_id"])
    np.testing.assert_array_equal(ob, G["sp_mask_outbbox"].astype(bool))
    np.testing.assert_array_equal(pts, G["sp_pts"])
    assert G["sp_mask_outbbox"].any() and not G["sp_mask_outbbox"].all()


def test_maskcache_exact(G):
    shape = tuple(int(s) for s in G["mc_shape"])
    world = np.unpackbits(G["mc_world"])[:int(np.prod(shape))].reshape(shape).astype(bool)
    out = O.maskcache(world, G["mc_xyz"], G["mc_scale"], G["mc_shift"])
    np.testing.assert_array_equal(out, G["mc_out"].astype(bool))


@pytest.mark.parametrize("tag,interval", [("05", 0.5), ("10", 1.0)])
def test_raw2alpha_ulps(G, tag, interval):
    shift = float(G["ra_params"][0])
    d = G["ra_density"]
    e, a = O.raw2alpha(d, shift, interval, fp32=True)
    re, ra = G[f"ra{tag}_exp"], G[f"ra{tag}_alpha"]
    fin = np.isfinite(re)
    np.testing.assert_array_equal(np.isfinite(e), fin)  # exp overflows exactly where it does
    assert _ulps(e[fin], re[fin]).max() <= 2
    # alpha = 1 - pow(..): an ulp of pow near 1 is 6e-8 absolute, whatever alpha is
    assert np.abs(a - ra).max() <= 4 * 2.0 ** -24
    # backward from the reference's own exp values: pow's last bit at most
    g = O.raw2alpha_backward(re, G[f"ra{tag}_grad_back"], interval, fp32=True)
    rg = G[f"ra{tag}_grad"]
    assert _ulps(np.abs(g), np.abs(rg)).max() <= 4
    assert np.array_equal(np.sign(g), np.sign(rg))


def test_alpha2weight_exact(G):
    n_rays = int(G["aw_n_rays"])
    rid = G["aw_ray_id"].astype(np.int64)
    w, T, last, i_s, i_e = O.alpha2weight(G["aw_alpha"], rid, n_rays, fp32=True)
    np.testing.assert_array_equal(i_s, G["aw_i_start"])
    np.testing.assert_array_equal(i_e, G["aw_i_end"])
    np.testing.assert_array_equal(np.float32(last), G["aw_last"])
    # T and weight are written only up to each ray's stop (zeros / ones after)
    np.testing.assert_array_equal(np.float32(T), G["aw_T"])
    np.testing.assert_array_equal(np.float32(w), G["aw_weight"])
    stopped = (G["aw_i_end"] < np.bincount(rid, minlength=n_rays).cumsum())
    assert stopped.sum() > 50 and (~stopped).sum() >= 10


def test_alpha2weight_backward_exact(G):
    g = O.alpha2weight_backward(G["aw_alpha"], G["aw_weight"], G["aw_T"], G["aw_last"],
                                G["aw_i_start"], G["aw_i_end"], G["aw_grad_weights"],
                                G["aw_grad_last"], fp32=True)
    np.testing.assert_array_equal(np.float32(g), G["aw_grad"])


@pytest.mark.parametrize("tag", ["c1d", "c1s", "c12s", "c12d"])
def test_tv_exact(G, tag):
    p = G[f"tv{tag}_param"][0]  # [C, X, Y, Z]
    C_, X, Y, Z = p.shape
    vals = np.moveaxis(p, 0, -1)
    act = np.ones((X, Y, Z), np.uint8)
    og = O.OGridData((X, Y, Z), vals, act, background=0.0)
    gin = np.moveaxis(G[f"tv{tag}_grad_in"][0], 0, -1)
    gp = O.OGridData((X, Y, Z), gin, act, background=0.0).p_values.copy()
    wx, wy, wz = (float(x) / 6 for x in G[f"tv{tag}_w"])
    wx, wy, wz = (float(np.float32(x)) for x in (wx, wy, wz))
    O.tv(og, gp, wx, wy, wz, int(G[f"tv{tag}_dense"]), fp32=True)
    got = np.moveaxis(og.unpad(gp), -1, 0)
    np.testing.assert_array_equal(np.float32(got), G[f"tv{tag}_grad_out"][0])


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_adam_dense_exact(G, mode):
    lr, b1, b2, eps = (float(x) for x in G["adam_params"])
    p = G[f"adam{mode}_p0"].astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    perlr = G[f"adam{mode}_perlr"] if mode == 2 else None
    for step in (1, 2, 3):
        p, m, v = O.adam_dense(p, G[f"adam{mode}_g{step}"], m, v, perlr, step, b1, b2, lr, eps,
                               mode, fp32=True)
        np.testing.assert_array_equal(np.float32(m), G[f"adam{mode}_m{step}"])
        np.testing.assert_array_equal(np.float32(v), G[f"adam{mode}_v{step}"])
        np.testing.assert_array_equal(np.float32(p), G[f"adam{mode}_p{step}"])
    if mode == 1:  # zero gradients leave their parameters untouched
        untouched = np.ones(p.size, bool)
        for step in (1, 2, 3):
            untouched &= G[f"adam1_g{step}"] == 0
        assert untouched.any()
        np.testing.assert_array_equal(G["adam1_p3"][untouched], G["adam1_p0"][untouched])
