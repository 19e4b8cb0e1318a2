"""ORACLE — test infrastructure only (tests/, bench.py's CPU baseline). Numpy
restatements of the DVGO schedule around the training step, in FP32 where the
reference computes in FP32 (every numpy float32 operation rounds once, like
the reference's separate torch kernels):

* merged-row compression        vdb_compression.py:24-58
* rescaling (align_corners)     lib/grid.py:91-102 (F.interpolate trilinear)
* occupancy builds               lib/dvgo.py:186-210, lib/grid.py:214-221
* near-camera masking           lib/dvgo.py:163-175
* per-view voxel counts         lib/dvgo.py:212-243 (grid_sample backward)
* pinhole / NDC rays            lib/dvgo.py:471-521
* hit_coarse_geo                lib/dvgo.py:258-270

The golden fixture tests/golden/lifecycle_golden.npz, generated by running the
reference's own functions (tests/golden/make_lifecycle_golden.py), pins these.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

f32 = np.float32


def norm3_f32(v):
    """torch's CPU vector norm of [...,3] float32: sqrt(fma(z,z,fma(y,y,x*x)))
    (the fused multiply-adds emulated in float64: exact products, one
    rounding each)."""
    x, y, z = (v[..., k].astype(np.float64) for k in range(3))
    inner = (y * y + (x * x).astype(f32).astype(np.float64)).astype(f32).astype(np.float64)
    return np.sqrt((z * z + inner).astype(f32)).astype(f32)


def linspace_f32(start, end, n):
    """torch.linspace in float32 by ATen's scalar two-sided formula: start +
    step*i for the first half, end - step*(n-1-i) for the second (ATen's
    vectorised CPU path can differ by one ulp of the range)."""
    start, end = f32(start), f32(end)
    if n == 1:
        return np.array([start], f32)
    step = f32((end - start) / f32(n - 1))
    i = np.arange(n)
    first = start + step * i.astype(f32)
    second = end - step * (n - 1 - i).astype(f32)
    return np.where(i < n // 2, first, second).astype(f32)


def grid_points(xyz_min, xyz_max, shape):
    """meshgrid(linspace per axis, indexing='ij') -> [X,Y,Z,3] float32."""
    lin = [linspace_f32(xyz_min[a], xyz_max[a], shape[a]) for a in range(3)]
    g = np.meshgrid(*lin, indexing="ij")
    return np.stack(g, -1).astype(f32)


# ------------------------------------------------------------------ merge
def merge(den, col, mask, dtype=np.float16):
    """(index [X,Y,Z] int32, den_rows [N+1], col_rows [N+1, C]): row ids 1..N
    of the masked voxels in C order, row 0 zero (vdb_compression.py:27-58)."""
    mask = np.asarray(mask).astype(bool)
    n = int(mask.sum())
    index = np.zeros(mask.shape, np.int32)
    index[mask] = np.arange(1, n + 1, dtype=np.int32)
    # values beyond the FP16 range become inf, as torch's .half() makes them
    with np.errstate(over="ignore"):
        den_rows = None if den is None else np.concatenate(
            [[0.0], np.asarray(den, np.float32)[mask]]).astype(np.float32).astype(dtype)
        col_rows = None
        if col is not None:
            col = np.asarray(col, np.float32)
            col_rows = np.concatenate([np.zeros((1, col.shape[-1]), np.float32),
                                       col[mask]]).astype(dtype)
    return index, den_rows, col_rows


# --------------------------------------------------------------- rescale
def _axis(in_size, out_size):
    scale = f32(f32(in_size - 1) / f32(out_size - 1)) if out_size > 1 else f32(0)
    real = (scale * np.arange(out_size).astype(f32)).astype(f32)
    i0 = np.minimum(np.floor(real).astype(np.int64), in_size - 1)
    l1 = np.clip(real - i0.astype(f32), f32(0), f32(1)).astype(f32)
    i1 = i0 + (i0 < in_size - 1)
    return i0, i1, (f32(1) - l1).astype(f32), l1


def resample(values, new_ws):
    """F.interpolate(mode='trilinear', align_corners=True) of values
    [X,Y,Z,C] (ATen upsample_trilinear3d): the z interpolation nested in y
    nested in x, each a*w0 + b*w1 evaluated as fma(a, w0, b*w1) like ATen's
    CPU build does for 1- and 3-channel volumes (some wider shapes take
    another ATen order, a few ulps apart). The fma is emulated in float64:
    the exact sum rounded once."""
    v = np.asarray(values, f32)
    ax = [_axis(v.shape[a], int(new_ws[a])) for a in range(3)]
    (x0, x1, wx0, wx1), (y0, y1, wy0, wy1), (z0, z1, wz0, wz1) = ax

    def at(xi, yi, zi):
        return v[xi][:, yi][:, :, zi]

    W = lambda w, s: w.reshape(s)  # noqa: E731
    wz0_, wz1_ = W(wz0, (1, 1, -1, 1)), W(wz1, (1, 1, -1, 1))
    wy0_, wy1_ = W(wy0, (1, -1, 1, 1)), W(wy1, (1, -1, 1, 1))
    wx0_, wx1_ = W(wx0, (-1, 1, 1, 1)), W(wx1, (-1, 1, 1, 1))

    def lerp(a, wa, b, wb):
        # fma(a, wa, b*wb): one rounding of the exact a*wa + round(b*wb)
        return (a.astype(np.float64) * wa + (b * wb).astype(f32).astype(np.float64)).astype(f32)

    def lz(xi, yi):
        return lerp(at(xi, yi, z0), wz0_, at(xi, yi, z1), wz1_)

    def ly(xi):
        return lerp(lz(xi, y0), wy0_, lz(xi, y1), wy1_)

    return lerp(ly(x0), wx0_, ly(x1), wx1_)


# ------------------------------------------------------------- occupancy
def maxpool3(a):
    """max_pool3d(kernel 3, padding 1, stride 1): padding never wins."""
    p = np.pad(a, 1, constant_values=-np.inf)
    X, Y, Z = a.shape
    out = np.full(a.shape, -np.inf, a.dtype)
    for dx in range(3):
        for dy in range(3):
            for dz in range(3):
                out = np.maximum(out, p[dx:dx + X, dy:dy + Y, dz:dz + Z])
    return out


def raw2alpha_f32(d, shift, interval):
    return O.raw2alpha(np.asarray(d, f32).reshape(-1), shift, interval, fp32=True)[1].astype(
        f32).reshape(np.shape(d))


def softplus_alpha(x, interval):
    """1 - exp(-softplus(x) * interval), softplus = log1p(exp(x)) with torch's
    threshold 20 (torch's vectorised CPU kernel uses log(exp(x) + 1))."""
    x = np.asarray(x, f32)
    sp = np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, f32(20))))).astype(f32)
    return (f32(1) - np.exp(-(sp * f32(interval)))).astype(f32)


def occupancy(mode, density: O.OGridData, shape, xyz_min, xyz_max, act_shift, interval, thres,
              mask=None, old_mask=None):
    """(mask [shape] bool, margin [shape]): the three mask-cache builds; the
    margin is the pooled value that was compared with the threshold (alpha),
    for telling apart the voxels that sit on the threshold."""
    shape = tuple(int(s) for s in shape)
    mn = np.asarray(xyz_min, f32)
    mx = np.asarray(xyz_max, f32)
    if mode == 0:
        pts = grid_points(mn, mx, shape).reshape(-1, 3)
        ws1 = np.array(density.reso, f32) - f32(1)
        idx = (((pts - mn) / (mx - mn)) * ws1).astype(f32)
        val = O.sample(density, idx, fp32=True)[:, 0].astype(f32)
        a = raw2alpha_f32(val, act_shift, interval).reshape(shape)
    else:
        dense = density.dense()[..., 0].astype(f32)
        a = raw2alpha_f32(dense, act_shift, interval) if mode == 1 else dense
    pooled = maxpool3(a)
    if mode == 0:
        return np.asarray(mask).astype(bool) & (pooled > f32(thres)), pooled
    if mode == 1:
        keep = pooled > f32(thres)
        if old_mask is not None:
            om = np.asarray(old_mask).astype(np.uint8)
            sc = ((np.array(om.shape, f32) - f32(1)) / (mx - mn)).astype(f32)
            sh = (-mn * sc).astype(f32)
            pts = grid_points(mn, mx, shape).reshape(-1, 3)
            keep &= O.maskcache(om, pts, sc, sh).reshape(shape)
        return keep, pooled
    alpha = softplus_alpha(pooled + f32(act_shift), interval)
    return alpha >= f32(thres), alpha


# --------------------------------------------------------- near cameras
def near_cam_mask(reso, cams, near_clip, xyz_min, xyz_max):
    """Grid points within near_clip of a camera centre (lib/dvgo.py:166-174)."""
    pts = grid_points(np.asarray(xyz_min, f32), np.asarray(xyz_max, f32), reso)
    best = np.full(tuple(reso), np.inf, f32)
    for c in np.asarray(cams, f32).reshape(-1, 3):
        d = pts - c
        dist = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
        best = np.minimum(best, dist.astype(f32))
    return best <= f32(near_clip)


# ----------------------------------------------------------- view counts
def view_weight_sums(rays_o, rays_d, reso, xyz_min, xyz_max, near, stepdist, n_samples):
    """Per-voxel sum (float64) of the trilinear weights of one view's samples
    (lib/dvgo.py:224-240 with grid_sample's zero padding)."""
    ro = np.asarray(rays_o, f32).reshape(-1, 3)
    rd = np.asarray(rays_d, f32).reshape(-1, 3)
    mn, mx = np.asarray(xyz_min, f32), np.asarray(xyz_max, f32)
    vec = np.where(rd == 0, f32(1e-6), rd).astype(f32)
    ra = ((mx - ro) / vec).astype(f32)
    rb = ((mn - ro) / vec).astype(f32)
    t_min = np.clip(np.minimum(ra, rb).max(-1), f32(near), f32(1e9)).astype(f32)
    step = (f32(stepdist) * np.arange(n_samples).astype(f32)).astype(f32)
    dn = norm3_f32(rd)
    t = (t_min[:, None] + step[None, :] / dn[:, None]).astype(f32)
    pts = (ro[:, None, :] + rd[:, None, :] * t[..., None]).astype(f32).reshape(-1, 3)
    nrm = ((((pts - mn) / (mx - mn)) * f32(2)) - f32(1)).astype(f32)
    g = (((nrm + f32(1)) * f32(0.5)) * (np.array(reso, f32) - f32(1))).astype(f32)
    g0 = np.floor(g)
    acc = np.zeros(tuple(reso), np.float64)
    for c in range(8):
        off = np.array([(c >> 2) & 1, (c >> 1) & 1, c & 1])
        idx = g0 + off
        w = np.where(off == 1, g - g0, (g0 + 1) - g).astype(f32)
        wt = (w[:, 2] * w[:, 1]) * w[:, 0]
        ok = np.all((idx >= 0) & (idx <= np.array(reso) - 1), axis=1) & (wt > 0)
        ii = idx[ok].astype(np.int64)
        np.add.at(acc, (ii[:, 0], ii[:, 1], ii[:, 2]), wt[ok].astype(np.float64))
    return acc


# ------------------------------------------------------------------ rays
def get_rays(H, W, K, c2w, inverse_y, flip_x, flip_y, mode="center", jitter=None, ndc=False):
    """(rays_o, rays_d, viewdirs) [H,W,3] float32 (lib/dvgo.py:471-521)."""
    K = np.asarray(K, np.float64).reshape(3, 3)
    fx, cx, fy, cy = f32(K[0, 0]), f32(K[0, 2]), f32(K[1, 1]), f32(K[1, 2])
    c2w = np.asarray(c2w, f32).reshape(-1, 4)
    i = np.broadcast_to(np.arange(W, dtype=f32)[None, :], (H, W)).astype(f32)
    j = np.broadcast_to(np.arange(H, dtype=f32)[:, None], (H, W)).astype(f32)
    if mode == "center":
        i, j = i + f32(0.5), j + f32(0.5)
    elif mode == "random":
        i, j = i + jitter[0], j + jitter[1]
    if flip_x:
        i = i[:, ::-1]
    if flip_y:
        j = j[::-1, :]
    d0 = (i - cx) / fx
    d1 = (j - cy) / fy if inverse_y else -((j - cy) / fy)
    d2 = np.full((H, W), f32(1) if inverse_y else f32(-1), f32)
    R = c2w[:3, :3]
    rd = np.stack([(d0 * R[k, 0] + d1 * R[k, 1]) + d2 * R[k, 2] for k in range(3)], -1).astype(f32)
    vd = (rd / norm3_f32(rd)[..., None]).astype(f32)
    ro = np.broadcast_to(c2w[:3, 3], rd.shape).astype(f32)
    if ndc:
        near = f32(1)
        ax = f32(-1.0 / (W / (2.0 * K[0, 0])))
        ay = f32(-1.0 / (H / (2.0 * K[0, 0])))
        t = (-(near + ro[..., 2]) / rd[..., 2]).astype(f32)
        ro = (ro + t[..., None] * rd).astype(f32)
        ox, oy, oz = ro[..., 0], ro[..., 1], ro[..., 2]
        dx, dy, dz = rd[..., 0], rd[..., 1], rd[..., 2]
        o_new = np.stack([(ax * ox) / oz, (ay * oy) / oz, f32(1) + f32(2) * near / oz], -1)
        d_new = np.stack([ax * (dx / dz - ox / oz), ay * (dy / dz - oy / oz),
                          (f32(-2) * near) / oz], -1)
        ro, rd = o_new.astype(f32), d_new.astype(f32)
    return ro, rd, vd


def hit_coarse_geo(rays_o, rays_d, xyz_min, xyz_max, near, stepdist, mask):
    """The reference's composition (lib/dvgo.py:265-269) over the oracle's
    sample_pts_on_rays and maskcache_lookup."""
    ro = np.asarray(rays_o, f32).reshape(-1, 3)
    rd = np.asarray(rays_d, f32).reshape(-1, 3)
    p = O.march_params(xyz_min, xyz_max, near, stepdist, 0.0, 1.0, 0.0, far=1e9)
    pts, ob, rid, _ = O.ray_points(ro, rd, p)
    mn, mx = np.asarray(xyz_min, f32), np.asarray(xyz_max, f32)
    m = np.asarray(mask).astype(np.uint8)
    sc = ((np.array(m.shape, f32) - f32(1)) / (mx - mn)).astype(f32)
    sh = (-mn * sc).astype(f32)
    inside = ~ob
    hit = np.zeros(ro.shape[0], bool)
    hit[rid[inside][O.maskcache(m, pts[inside], sc, sh)]] = True
    return hit
