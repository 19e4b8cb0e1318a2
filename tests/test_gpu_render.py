"""GPU parity of the merged-index renderer (MGRenderer, renderer.cu:122-412)
against the CPU oracle: the FP32 path against the float-mirroring oracle and
against FP64 (RGB within 1e-5 relative), the BF16 path (BF16 features, BF16
rgbnet on the tensor cores) against FP64, and determinism."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RESO = 48
HW = 96


@pytest.fixture(scope="module")
def scene(lib):
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, rgbnet_init, scene_dense, sphere_poses
    from plenvdb_gb300.trainer import FineStageConfig
    scfg = SceneConfig(reso=RESO, n_ellipsoids=6, seed=21)
    cfg = FineStageConfig(reso=RESO)
    cam = CameraConfig()
    active, dens, k0 = scene_dense(scfg)
    active = active.astype(bool)
    n = int(active.sum())
    index = np.zeros(active.shape, np.int32)
    index[active] = np.arange(1, n + 1, dtype=np.int32)
    # raw density N(5,1): alpha ~0.4 per sample, so the T < t_stop stop is exercised
    den = np.concatenate([[0.0], dens[active] + 3.0]).astype(np.float32)
    col = np.concatenate([np.zeros((1, 12)), k0[active]]).astype(np.float32)
    net = [t.numpy().astype(np.float64) for t in rgbnet_init(seed=3)]
    f = cam.focal * HW / cam.W
    K = np.array([[f, 0, HW / 2], [0, f, HW / 2], [0, 0, 1]], np.float32)
    poses = sphere_poses(3, cam.radius, seed=5)
    return dict(scfg=scfg, cfg=cfg, cam=cam, index=index, den=den, col=col, net=net, K=K,
                poses=poses)


def _kw(s, t_stop):
    c = s["cfg"]
    return dict(near=s["cam"].near, stepdist=c.stepdist, act_shift=c.act_shift,
                interval=c.interval, thres=c.fast_color_thres, bg=1.0, t_stop=t_stop)


def _gpu_render(s, pose, storage, precision, t_stop):
    from plenvdb_gb300.renderer import MGRenderer
    c, kw = s["cfg"], _kw(s, t_stop)
    r = MGRenderer(12, 27, 128, 3)
    r.load_data(s["den"], s["col"], s["index"], s["den"].shape[0], storage=storage)
    w0, b0, w1, b1, w2, b2 = s["net"]
    r.load_params(w0.T.copy(), b0, w1.T.copy(), b1, w2.T.copy(), b2)  # reference layout [in,out]
    r.setScene([RESO] * 3, s["K"], c.xyz_min, c.xyz_max)
    r.setKwargs(kw["near"], 1e9, kw["stepdist"], kw["act_shift"], kw["interval"], kw["thres"],
                kw["bg"], False, HW, HW, t_stop=t_stop)
    r.precision = precision
    r.input_a_c2w(pose)
    r.render_an_image()
    return r.output_an_image().reshape(-1, 3).astype(np.float64)


def _oracle_render(s, pose, t_stop, fp32, col=None):
    c = s["cfg"]
    mlp = O.MLPWeights(*s["net"], c0=12, pe=4)
    rgb, ncol, _ = O.render_pixels(s["index"], s["den"], s["col"] if col is None else col, mlp,
                                   s["K"], pose, c.xyz_min, c.xyz_max, HW, HW, fp32=fp32,
                                   **_kw(s, t_stop))
    return rgb, ncol


@pytest.mark.parametrize("t_stop", [1e-3, 1e-4])
def test_render_fp32_matches_oracle(scene, t_stop):
    s = scene
    for pose in s["poses"][:2]:
        img = _gpu_render(s, pose, 0, 0, t_stop)
        o32, ncol = _oracle_render(s, pose, t_stop, fp32=True)
        o64, _ = _oracle_render(s, pose, t_stop, fp32=False)
        assert (ncol > 0).mean() > 0.2, "the view should cover the scene"
        # pixels without a colour sample are the background exactly
        empty = ncol == 0
        assert np.array_equal(img[empty], np.ones_like(img[empty]))
        # float-mirroring oracle: equal up to libm ulps, except where a libm ulp
        # flips a threshold decision (a handful of pixels at most)
        far32 = np.abs(img - o32).max(axis=1) > 1e-5
        assert far32.mean() <= 0.01, f"{far32.sum()} pixels off the fp32 oracle"
        # FP64 truth: 1e-5 relative on all but threshold-flip pixels
        rel = np.abs(img - o64) / np.maximum(np.abs(o64), 1e-3)
        bad = rel.max(axis=1) > 1e-5
        assert bad.mean() <= 0.01, f"{bad.sum()} pixels beyond 1e-5 relative of FP64"
        assert np.median(rel) < 1e-6


def test_render_bf16_within_tolerance_of_fp64(scene):
    s = scene
    pose = s["poses"][2]
    img = _gpu_render(s, pose, 1, 1, 1e-4)
    o64, ncol = _oracle_render(s, pose, 1e-4, fp32=False)
    err = np.abs(img - o64).max(axis=1)
    hit = ncol > 0
    assert err[~hit].max() == 0.0
    # BF16 features (8-bit mantissa) and BF16 rgbnet operands with FP32 accumulation
    assert err[hit].mean() < 5e-3, err[hit].mean()
    assert np.quantile(err[hit], 0.99) < 3e-2, np.quantile(err[hit], 0.99)
    # against the same features rounded to BF16 the remaining error is the
    # rgbnet's (BF16 operands, FP32 accumulation)
    import torch
    colb = torch.from_numpy(s["col"]).to(torch.bfloat16).float().numpy()
    o64b, _ = _oracle_render(s, pose, 1e-4, fp32=False, col=colb)
    errb = np.abs(img - o64b).max(axis=1)
    assert errb[hit].mean() < 5e-3, errb[hit].mean()


def test_render_deterministic_and_storage_agrees(scene):
    s = scene
    pose = s["poses"][0]
    a = _gpu_render(s, pose, 0, 0, 1e-3)
    b = _gpu_render(s, pose, 0, 0, 1e-3)
    assert np.array_equal(a, b)
    c = _gpu_render(s, pose, 0, 1, 1e-3)   # BF16 rgbnet on FP32 features
    d = _gpu_render(s, pose, 1, 0, 1e-3)   # FP32 rgbnet on BF16 features
    assert np.abs(c - a).max() < 5e-2 and np.abs(d - a).max() < 5e-2
