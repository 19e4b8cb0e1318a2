"""The lifecycle oracle's floating-point building blocks against the torch CPU
operations the reference calls, over random shapes (beyond the golden
fixture's cases):

* max_pool3d(3, padding 1) and the vector norm: bit-exact;
* F.interpolate(trilinear, align_corners=True): bit-exact for 1- and 3-channel
  volumes; ATen evaluates some 12-channel shapes in another order, within a
  few ulps;
* torch.linspace: within one ulp of the range (ATen's vectorised path splits
  the two-sided formula into chunks whose bases round differently, by CPU);
* 1 - exp(-softplus(x) * interval): within 2e-5 relative, or a couple of
  ulps of 1.0 for tiny alphas (torch's vectorised CPU softplus forms
  log(exp(x) + 1), its scalar path and the oracle log1p).
CPU only."""
import numpy as np
import torch
import torch.nn.functional as F

from oracle import lifecycle as OL


def test_maxpool_bit_exact():
    rng = np.random.default_rng(0)
    for _ in range(10):
        s = tuple(int(x) for x in rng.integers(1, 20, 3))
        a = rng.normal(size=s).astype(np.float32)
        ref = F.max_pool3d(torch.from_numpy(a)[None, None], kernel_size=3, padding=1, stride=1)
        np.testing.assert_array_equal(OL.maxpool3(a), ref[0, 0].numpy())


def test_norm_bit_exact():
    v = np.random.default_rng(1).normal(size=(100000, 3)).astype(np.float32)
    np.testing.assert_array_equal(OL.norm3_f32(v), torch.from_numpy(v).norm(dim=-1).numpy())


def test_resample_against_interpolate():
    rng = np.random.default_rng(2)
    for _ in range(24):
        src = tuple(int(x) for x in rng.integers(2, 20, 3))
        dst = tuple(int(x) for x in rng.integers(1, 30, 3))
        C = int(rng.choice([1, 3, 12]))
        v = rng.normal(size=src + (C,)).astype(np.float32)
        ref = F.interpolate(torch.from_numpy(v).permute(3, 0, 1, 2)[None], size=dst,
                            mode="trilinear", align_corners=True)[0].permute(1, 2, 3, 0).numpy()
        out = OL.resample(v, dst)
        if C < 12:
            np.testing.assert_array_equal(out, ref, err_msg=str((src, dst, C)))
        else:
            np.testing.assert_allclose(out, ref, rtol=0, atol=8 * 2.0 ** -23 * np.abs(v).max())


def test_linspace_within_one_ulp_of_the_range():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 7, 8, 9, 16, 17, 33, 64, 65, 160, 257, 320):
        a, b = np.float32(rng.uniform(-3, 0)), np.float32(rng.uniform(0, 3))
        ref = torch.linspace(float(a), float(b), n).numpy()
        out = OL.linspace_f32(a, b, n)
        assert out.dtype == np.float32 and out.shape == ref.shape
        np.testing.assert_allclose(out, ref, rtol=0, atol=2.0 ** -22 * max(abs(a), abs(b)))


def test_softplus_alpha_against_torch():
    x = np.random.default_rng(4).normal(0, 8, 100000).astype(np.float32)
    ref = (1 - torch.exp(-F.softplus(torch.from_numpy(x)) * 0.5)).numpy()
    out = OL.softplus_alpha(x, 0.5)
    # 1 - exp(-y) is formed next to 1.0 in FP32 on both sides: tiny alphas
    # agree to a couple of ulps of 1.0, the rest to 2e-5 relative
    np.testing.assert_allclose(out, ref, rtol=2e-5, atol=2.5e-7)
