"""The standalone DirectVoxGO primitives (plenvdb_gb300.render_utils, the
render_utils_cuda replacement) against the oracle's restatement of the
reference kernels (render_utils_kernel.cu): ray sampling and the mask cache
exactly, raw2alpha / alpha2weight and their backward within libm ulps (the
oracle's FP32 mode keeps the reference's double products; the GPU path is
FP32 only). Includes rays that miss the bbox and empty inputs."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rays(lib):
    from plenvdb_gb300.scene import CameraConfig, random_rays
    ro, rd, vd = random_rays(CameraConfig(), 300, 5, seed=31)
    # a few rays that miss the bbox entirely, and one along an axis (d_x = 0)
    ro[:4] = np.array([5.0, 5.0, 5.0], np.float32)
    rd[:4] = np.array([0.3, 0.5, 0.8], np.float32)
    rd[4] = np.array([0.0, 0.0, -1.0], np.float32)
    ro[4] = np.array([0.2, -0.3, 4.0], np.float32)
    return ro, rd


def test_sample_pts_on_rays_exact(rays):
    import torch
    from plenvdb_gb300 import render_utils as RU
    ro, rd = rays
    lo, hi = [-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]
    near, far, step = 2.0, 1e9, 0.5 * 3.0 / 160
    pts, ob, rid, sid, ns, tmin, tmax = RU.sample_pts_on_rays(
        torch.from_numpy(ro).cuda(), torch.from_numpy(rd).cuda(), torch.tensor(lo),
        torch.tensor(hi), near, far, step)
    p = O.march_params(lo, hi, near, step, -4.6, 0.5, 1e-4, far=far)
    otmin, otmax, ons = O.ray_count(ro, rd, p)
    opts, oob, orid, osid = O.ray_points(ro, rd, p)
    np.testing.assert_array_equal(tmin.cpu().numpy(), otmin)
    np.testing.assert_array_equal(tmax.cpu().numpy(), otmax)
    np.testing.assert_array_equal(ns.cpu().numpy(), ons)
    np.testing.assert_array_equal(rid.cpu().numpy(), orid)
    np.testing.assert_array_equal(sid.cpu().numpy(), osid)
    np.testing.assert_array_equal(ob.cpu().numpy(), oob)
    np.testing.assert_array_equal(pts.cpu().numpy(), opts)
    assert ns.min().item() >= 1  # N_steps = max(ceil(...), 1), also for rays that miss


def test_maskcache_lookup_exact(rays, lib):
    import torch
    from plenvdb_gb300 import render_utils as RU
    rng = np.random.default_rng(5)
    world = rng.random((33, 40, 27)) < 0.3
    xyz = rng.uniform(-1.8, 1.8, (5000, 3)).astype(np.float32)
    xyz[:50] = np.round(xyz[:50] * 10) / 10  # values on the rounding boundaries
    scale = ((np.array(world.shape) - 1) / 3.0).astype(np.float32)
    shift = (1.5 * scale).astype(np.float32)
    out = RU.maskcache_lookup(torch.from_numpy(world).cuda(), torch.from_numpy(xyz).cuda(),
                              torch.from_numpy(scale), torch.from_numpy(shift))
    ref = O.maskcache(world, xyz, scale, shift)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_raw2alpha_and_backward(lib):
    import torch
    from plenvdb_gb300 import render_utils as RU
    rng = np.random.default_rng(6)
    d = rng.normal(0, 4, 20000).astype(np.float32)
    d[:4] = [-100.0, 100.0, 0.0, 4.6]
    e, a = RU.raw2alpha(torch.from_numpy(d).cuda(), -4.6, 0.5)
    oe, oa = O.raw2alpha(d, -4.6, 0.5, fp32=True)
    np.testing.assert_allclose(e.cpu().numpy(), oe, rtol=2e-6, atol=0)
    np.testing.assert_allclose(a.cpu().numpy(), oa, rtol=2e-6, atol=1e-7)
    g = rng.normal(0, 1, d.size).astype(np.float32)
    gd = RU.raw2alpha_backward(e, torch.from_numpy(g).cuda(), 0.5)
    ogd = O.raw2alpha_backward(oe, g, 0.5, fp32=True)
    np.testing.assert_allclose(gd.cpu().numpy(), ogd, rtol=1e-5, atol=1e-30)
    # empty input
    e0, a0 = RU.raw2alpha(torch.zeros(0, device="cuda"), -4.6, 0.5)
    assert e0.numel() == 0 and a0.numel() == 0


def test_alpha2weight_and_backward(lib):
    import torch
    from plenvdb_gb300 import render_utils as RU
    rng = np.random.default_rng(7)
    n_rays = 200
    counts = rng.integers(0, 60, n_rays)
    counts[:3] = 0  # rays without points
    ray_id = np.repeat(np.arange(n_rays), counts).astype(np.int64)
    alpha = rng.beta(0.5, 2.0, ray_id.size).astype(np.float32)
    alpha[::37] = 0.999  # push some rays below the T < 1e-3 stop
    w, T, last, i_s, i_e = RU.alpha2weight(torch.from_numpy(alpha).cuda(),
                                           torch.from_numpy(ray_id).cuda(), n_rays)
    ow, oT, olast, ois, oie = O.alpha2weight(alpha, ray_id, n_rays, fp32=True)
    np.testing.assert_array_equal(i_s.cpu().numpy(), ois)
    np.testing.assert_array_equal(i_e.cpu().numpy(), oie)
    np.testing.assert_allclose(w.cpu().numpy(), ow, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(T.cpu().numpy(), oT, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(last.cpu().numpy(), olast, rtol=1e-6, atol=1e-9)
    gw = rng.normal(0, 1, ray_id.size).astype(np.float32)
    gl = rng.normal(0, 1, n_rays).astype(np.float32)
    g = RU.alpha2weight_backward(torch.from_numpy(alpha).cuda(), w, T, last, i_s, i_e, n_rays,
                                 torch.from_numpy(gw).cuda(), torch.from_numpy(gl).cuda())
    og = O.alpha2weight_backward(alpha, ow, oT, olast, ois, oie, gw, gl, fp32=True)
    scale = np.abs(og).max()
    np.testing.assert_allclose(g.cpu().numpy(), og, rtol=1e-5, atol=1e-6 * scale)
