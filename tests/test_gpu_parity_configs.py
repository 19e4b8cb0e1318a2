"""CUDA-vs-oracle parity at the measured workloads, not only on toy scenes:

* the fine-stage bench scene: 160^3 grid, 8 seeded ellipsoids, the seeded
  8192-ray batch the bench times (FP32 plain path);
* the large scene: 320^3 grid, 32 ellipsoids + a thin shell, a seeded
  1024-ray subset of the 65536-ray batches (ragged counts up to ~1100 samples
  per ray).

Per scene:
* structure exact against the oracle's FP32 mode (the reference's float
  arithmetic): colour-row ray and step ids, per-ray kept and colour counts;
* values within 1e-5 relative of the FP64 oracle: alphainv_last, weights,
  k0 rows, rgbnet rgb and rgb_marched (weights of alphas at the 1e-4
  threshold get an absolute floor of 1e-7: the reference's own FP32 alpha,
  1 - powf(..), cancels there);
* one backward within 1e-4 of FP64: density and k0 voxel gradients for seeded
  upstream gradients.
A ray whose kept-sample structure differs between FP32 and FP64 (an alpha or
weight within rounding of a threshold) cannot be compared value by value;
those rays are counted (a handful at most) and the FP64 comparisons run over
the rest, with the GPU re-run on exactly that ray set."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _scene(reso, n_ell, shell, n_rays, ray_seed, subset=None):
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import march_params
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays, scene_mask
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=reso, n_ellipsoids=n_ell, shell=shell, seed=0)
    cfg = FineStageConfig(reso=reso)
    ro, rd, vd = random_rays(CameraConfig(), n_rays, 100, seed=ray_seed)
    if subset is not None:
        pick = np.random.default_rng(5).choice(n_rays, subset, replace=False)
        ro, rd, vd = ro[pick], rd[pick], vd[pick]
    dg, kg = build_grids(scfg)
    active = scene_mask(scfg)
    R3 = (reso,) * 3
    # the oracle reads the very values the GPU grids hold
    dens = dg.get_dense_grid().reshape(R3)
    k0 = kg.get_dense_grid().reshape(R3 + (12,))
    og = O.OGridData(R3, dens, active, background=scfg.background)
    ok = O.OGridData(R3, k0, active, background=0.0)
    del k0
    op = O.march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                        cfg.interval, cfg.fast_color_thres)
    gp = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist, cfg.act_shift,
                      cfg.interval, cfg.fast_color_thres)
    return dict(scfg=scfg, cfg=cfg, ro=ro, rd=rd, vd=vd, dg=dg, kg=kg, og=og, ok=ok, op=op,
                gp=gp, reso=reso)


@pytest.fixture(scope="module")
def bench_scene(lib):
    return _scene(160, 8, False, 8192, 1)


@pytest.fixture(scope="module")
def large_scene(lib):
    return _scene(320, 32, True, 2 * 65536, 21, subset=1024)


def _gpu_march(s, sel=None):
    import torch
    from plenvdb_gb300.march import MarchSample, MarchWorkspace
    ro, rd = (s["ro"], s["rd"]) if sel is None else (s["ro"][sel], s["rd"][sel])
    ws = MarchWorkspace(max(ro.shape[0], 1), s["cfg"].xyz_min, s["cfg"].xyz_max,
                        s["cfg"].stepdist)
    dummy = torch.zeros(1, device="cuda", requires_grad=True)
    out = MarchSample.apply(dummy, ws, s["dg"], s["kg"], torch.from_numpy(ro).cuda(),
                            torch.from_numpy(rd).cuda(), s["gp"])
    torch.cuda.synchronize()
    return ws, dummy, out


def _per_ray_steps(ray_id, step_id, R):
    out = [[] for _ in range(R)]
    for r, k in zip(ray_id.tolist(), step_id.tolist()):
        out[r].append(k)
    return out


def _agreeing_rays(o32, o64, R):
    """Rays whose kept and colour structure is the same in FP32 and FP64."""
    a = _per_ray_steps(o32.ray_id, o32.step_id, R)
    b = _per_ray_steps(o64.ray_id, o64.step_id, R)
    same = np.array([a[r] == b[r] for r in range(R)]) & (o32.n_kept == o64.n_kept)
    return same


def _check_structure(s):
    ws, _, (w, last, k0, rid) = _gpu_march(s)
    o32 = O.March(s["og"], s["ok"], s["ro"], s["rd"], s["op"], fp32=True)
    R = s["ro"].shape[0]
    assert o32.M > R  # a colour-row-rich batch
    np.testing.assert_array_equal(rid.cpu().numpy(), o32.ray_id)
    v = ws.rows(o32.M, 12)
    np.testing.assert_array_equal(v["step_id"].cpu().numpy(), o32.step_id)
    np.testing.assert_array_equal(v["n_color"].cpu().numpy(), o32.n_color)
    kept, rows, _ = ws.stats()
    assert (kept, rows) == (o32.K, o32.M)
    # the float arithmetic is the reference's; CUDA's and the host's libm may
    # differ in the last bit of expf/powf
    np.testing.assert_allclose(last.detach().cpu().numpy(), o32.T_last, rtol=2e-6, atol=0)
    np.testing.assert_allclose(w.detach().cpu().numpy(), o32.weight, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(k0.detach().cpu().numpy(), o32.k0, rtol=1e-6, atol=1e-7)
    return o32


def _check_fp64(s, o32):
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import CompositeFn, RgbNetFn
    from plenvdb_gb300.scene import rgbnet_init
    R = s["ro"].shape[0]
    o64 = O.March(s["og"], s["ok"], s["ro"], s["rd"], s["op"], fp32=False)
    same = _agreeing_rays(o32, o64, R)
    assert (~same).sum() <= max(4, R // 500), f"{(~same).sum()} rays differ in structure"
    sel = np.nonzero(same)[0]
    s_sel = dict(s, ro=s["ro"][sel], rd=s["rd"][sel], vd=s["vd"][sel])
    ws, dummy, (w, last, k0, rid) = _gpu_march(s_sel)
    o = O.March(s["og"], s["ok"], s_sel["ro"], s_sel["rd"], s["op"], fp32=False)
    assert o.M == w.shape[0]
    np.testing.assert_array_equal(rid.cpu().numpy(), o.ray_id)
    # the FP32 transmittance product (one rounding per kept sample, as the
    # reference's float chain) against FP64, on the longest chains of the batch
    T = last.detach().cpu().numpy().astype(np.float64)
    rel_T = np.abs(T - o.T_last) / np.maximum(np.abs(o.T_last), 1e-30)
    wv = w.detach().cpu().numpy().astype(np.float64)
    rel_w = np.abs(wv - o.weight) / np.maximum(np.abs(o.weight), 1e-30)
    print(f"FP32 vs FP64 over {o.R} rays, up to {int(o.n_kept.max())} kept samples per ray: "
          f"max rel err alphainv_last {rel_T.max():.3e}, weights (weight > 1e-3) "
          f"{rel_w[o.weight > 1e-3].max():.3e}")
    np.testing.assert_allclose(last.detach().cpu().numpy(), o.T_last, rtol=1e-5, atol=0)
    np.testing.assert_allclose(w.detach().cpu().numpy(), o.weight, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(k0.detach().cpu().numpy(), o.k0, rtol=1e-5, atol=1e-7)
    # rgbnet (FP32 plain path) and composite against FP64
    net = rgbnet_init(seed=3)
    mlp = O.MLPWeights(*[t.numpy().astype(np.float64) for t in net], c0=12, pe=4)
    rgb64 = o.rgb(mlp, s_sel["vd"])
    rgbm64 = o.composite(rgb64, 1.0)
    params = [t.cuda().requires_grad_() for t in net]
    vd = torch.from_numpy(s_sel["vd"]).cuda()
    rgb = RgbNetFn.apply(k0, vd, ws, 4, 0, *params)
    rgbm = CompositeFn.apply(w, rgb, last, ws, 1.0)
    np.testing.assert_allclose(rgb.detach().cpu().numpy(), rgb64, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(rgbm.detach().cpu().numpy(), rgbm64, rtol=1e-5, atol=1e-6)
    # one backward: seeded upstream gradients of the sample stage's outputs
    rng = np.random.default_rng(12)
    gw = rng.normal(0, 1, o.M).astype(np.float32)
    gl = rng.normal(0, 1, o.R).astype(np.float32)
    gk = rng.normal(0, 1, (o.M, 12)).astype(np.float32)
    s["dg"].zero_grad()
    s["kg"].zero_grad()
    torch.autograd.backward([w, last, k0], [torch.from_numpy(a).cuda() for a in (gw, gl, gk)])
    torch.cuda.synchronize()
    R3 = (s["reso"],) * 3
    gd = s["dg"].get_dense_grid(which=L.WHICH_GRAD).reshape(R3)
    ref_d, ref_k = o.backward_sample(gw, gl, gk)
    # compared where either side is nonzero (the rest of the grid is zero on both)
    nz = (ref_d != 0) | (gd != 0)
    sd = np.abs(ref_d).max()
    np.testing.assert_allclose(gd[nz], ref_d[nz], rtol=1e-4, atol=1e-4 * sd)
    del gd, ref_d, nz
    gkk = s["kg"].get_dense_grid(which=L.WHICH_GRAD).reshape(R3 + (12,))
    nz = (ref_k != 0) | (gkk != 0)
    sk = np.abs(ref_k).max()
    np.testing.assert_allclose(gkk[nz], ref_k[nz], rtol=1e-4, atol=1e-5 * sk)
    s["dg"].zero_grad()
    s["kg"].zero_grad()
    return int((~same).sum())


def test_bench_scene_structure_exact(bench_scene):
    o32 = _check_structure(bench_scene)
    bench_scene["o32"] = o32


def test_bench_scene_fp64(bench_scene):
    o32 = bench_scene.get("o32") or O.March(bench_scene["og"], bench_scene["ok"],
                                            bench_scene["ro"], bench_scene["rd"],
                                            bench_scene["op"], fp32=True)
    n_diff = _check_fp64(bench_scene, o32)
    print(f"160^3 / 8192 rays: {n_diff} rays differ in FP32/FP64 structure")


def test_large_scene_structure_exact(large_scene):
    o32 = _check_structure(large_scene)
    large_scene["o32"] = o32
    # the subset holds long, ragged rays
    _, _, ns = O.ray_count(large_scene["ro"], large_scene["rd"], large_scene["op"])
    assert ns.max() > 900 and ns.min() < 400


def test_large_scene_fp64(large_scene):
    o32 = large_scene.get("o32") or O.March(large_scene["og"], large_scene["ok"],
                                            large_scene["ro"], large_scene["rd"],
                                            large_scene["op"], fp32=True)
    n_diff = _check_fp64(large_scene, o32)
    print(f"320^3 / 1024 rays: {n_diff} rays differ in FP32/FP64 structure")
