"""Training rays (lib/dvgo.py:471-635) on libpvdb's CUDA kernels: the pinhole
rays of a view (``get_rays``, ``get_rays_of_a_view`` with the NDC warp), the
three training-ray gatherers of run.py (``get_training_rays``,
``get_training_rays_flatten``, ``get_training_rays_in_maskcache_sampling``,
which keeps the rays for which ``hit_coarse_geo`` finds an occupied mask-cache
voxel), and ``batch_indices_generator``. Same names, arguments and returns as
the reference; the outputs are CUDA tensors.

``model`` arguments need ``xyz_min``, ``xyz_max``, ``voxel_size`` and a
``mask_cache`` (``plenvdb_gb300.lifecycle.MaskGrid``)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L


def _K(K):
    k = K.detach().cpu().numpy() if torch.is_tensor(K) else np.asarray(K)
    return L.f64arr(np.asarray(k, np.float64).reshape(-1))


def _c2w(c2w):
    a = c2w.detach().float().cpu().numpy() if torch.is_tensor(c2w) else np.asarray(c2w, np.float32)
    a = np.asarray(a, np.float32)
    if a.shape[0] == 3:  # [3,4] pose
        a = np.concatenate([a.reshape(3, 4), np.array([[0, 0, 0, 1]], np.float32)])
    return L.f32arr(a.reshape(-1)[:16])


_MODES = {"center": 0, "lefttop": 1, "random": 2}


def _rays(H, W, K, c2w, ndc, inverse_y, flip_x, flip_y, mode, generator=None):
    H, W = int(H), int(W)
    n = H * W
    o = torch.empty(n, 3, device="cuda", dtype=torch.float32)
    d = torch.empty_like(o)
    v = torch.empty_like(o)
    if mode not in _MODES:
        raise NotImplementedError(mode)
    jitter = None
    if mode == "random":
        # torch.rand_like(i), torch.rand_like(j): i and j are expanded meshgrid
        # views, so each draw is a fresh row-major [H, W] tensor
        ji = torch.rand(H, W, generator=generator)
        jj = torch.rand(H, W, generator=generator)
        jitter = torch.cat([ji.reshape(-1), jj.reshape(-1)]).cuda()
    L.call("pvdb_get_rays", H, W, _K(K), _c2w(c2w), int(bool(ndc)), int(bool(inverse_y)),
           int(bool(flip_x)), int(bool(flip_y)), _MODES[mode], L.ptr(jitter), L.ptr(o), L.ptr(d),
           L.ptr(v), L.stream_of())
    return o.view(H, W, 3), d.view(H, W, 3), v.view(H, W, 3)


def get_rays(H, W, K, c2w, inverse_y, flip_x, flip_y, mode="center", generator=None):
    """(rays_o, rays_d) [H,W,3] (lib/dvgo.py:471-495)."""
    o, d, _ = _rays(H, W, K, c2w, False, inverse_y, flip_x, flip_y, mode, generator)
    return o, d


def get_rays_of_a_view(H, W, K, c2w, ndc, inverse_y, flip_x, flip_y, mode="center",
                       generator=None):
    """(rays_o, rays_d, viewdirs) [H,W,3] (lib/dvgo.py:517-521)."""
    return _rays(H, W, K, c2w, ndc, inverse_y, flip_x, flip_y, mode, generator)


@torch.no_grad()
def hit_coarse_geo(rays_o, rays_d, near, far, stepsize, *, xyz_min, xyz_max, voxel_size,
                   mask_cache, **render_kwargs):
    """Bool [rays.shape[:-1]]: some sample of the ray lies in an occupied voxel
    of the mask cache (lib/dvgo.py:258-270; far is 1e9 as in the reference)."""
    shape = rays_o.shape[:-1]
    ro = rays_o.reshape(-1, 3).to(device="cuda", dtype=torch.float32).contiguous()
    rd = rays_d.reshape(-1, 3).to(device="cuda", dtype=torch.float32).contiguous()
    hit = torch.empty(ro.shape[0], device="cuda", dtype=torch.uint8)
    stepdist = float(np.float32(stepsize) * np.float32(voxel_size))
    L.call("pvdb_rays_hit_mask", L.ptr(ro), L.ptr(rd), ro.shape[0], L.f32arr(_f3(xyz_min)),
           L.f32arr(_f3(xyz_max)), float(near), stepdist, L.ptr(mask_cache.mask),
           L.i32arr(list(mask_cache.mask.shape)), L.ptr(hit), L.stream_of())
    return hit.bool().reshape(shape)


def _f3(v):
    if torch.is_tensor(v):
        v = v.detach().float().cpu().numpy()
    return [float(x) for x in np.asarray(v, np.float32).reshape(-1)]


def _compact(keep, srcs, cap):
    """Stable compaction of [n,3] CUDA arrays by a uint8 flag (libpvdb)."""
    keep = keep.reshape(-1).to(torch.uint8).contiguous()
    srcs = [s.reshape(-1, 3).contiguous() for s in srcs]
    dsts = [torch.empty(cap, 3, device="cuda", dtype=torch.float32) for _ in srcs]
    n = C.c_int64()
    L.call("pvdb_compact_rows", L.ptr(keep), keep.numel(), L.ptrarr([L.ptr(s) for s in srcs]),
           L.ptrarr([L.ptr(d) for d in dsts]), len(srcs), cap, C.byref(n), L.stream_of())
    return [d[:n.value] for d in dsts], n.value


@torch.no_grad()
def get_training_rays(rgb_tr, train_poses, HW, Ks, ndc, inverse_y, flip_x, flip_y):
    """(rgb_tr, rays_o_tr, rays_d_tr, viewdirs_tr, imsz) with [n,H,W,3] rays (lib/dvgo.py:524-548)."""
    # one image size and one camera for all views, as the reference asserts
    assert len(np.unique(np.asarray(HW), axis=0)) == 1
    Kn = np.stack([np.asarray(k.cpu() if torch.is_tensor(k) else k, np.float64) for k in Ks])
    assert len(np.unique(Kn.reshape(len(Kn), -1), axis=0)) == 1
    assert len(rgb_tr) == len(train_poses) == len(Ks) == len(HW)
    H, W = (int(v) for v in np.asarray(HW)[0])
    K = Ks[0]
    n = len(rgb_tr)
    rays_o_tr = torch.zeros([n, H, W, 3], device="cuda")
    rays_d_tr = torch.zeros_like(rays_o_tr)
    viewdirs_tr = torch.zeros_like(rays_o_tr)
    for i, c2w in enumerate(train_poses):
        o, d, v = get_rays_of_a_view(H, W, K, c2w, ndc, inverse_y, flip_x, flip_y)
        rays_o_tr[i].copy_(o)
        rays_d_tr[i].copy_(d)
        viewdirs_tr[i].copy_(v)
    return rgb_tr, rays_o_tr, rays_d_tr, viewdirs_tr, [1] * n


@torch.no_grad()
def get_training_rays_flatten(rgb_tr_ori, train_poses, HW, Ks, ndc, inverse_y, flip_x, flip_y):
    """Flattened [N,3] rays of all views (lib/dvgo.py:551-579)."""
    assert len(rgb_tr_ori) == len(train_poses) == len(Ks) == len(HW)
    N = sum(im.shape[0] * im.shape[1] for im in rgb_tr_ori)
    rgb_tr = torch.zeros([N, 3], device="cuda")
    rays_o_tr = torch.zeros_like(rgb_tr)
    rays_d_tr = torch.zeros_like(rgb_tr)
    viewdirs_tr = torch.zeros_like(rgb_tr)
    imsz, top = [], 0
    for c2w, img, (H, W), K in zip(train_poses, rgb_tr_ori, HW, Ks):
        assert tuple(img.shape[:2]) == (int(H), int(W))
        o, d, v = get_rays_of_a_view(int(H), int(W), K, c2w, ndc, inverse_y, flip_x, flip_y)
        n = int(H) * int(W)
        rgb_tr[top:top + n].copy_(torch.as_tensor(img).reshape(-1, 3))
        rays_o_tr[top:top + n].copy_(o.reshape(-1, 3))
        rays_d_tr[top:top + n].copy_(d.reshape(-1, 3))
        viewdirs_tr[top:top + n].copy_(v.reshape(-1, 3))
        imsz.append(n)
        top += n
    return rgb_tr, rays_o_tr, rays_d_tr, viewdirs_tr, imsz


@torch.no_grad()
def get_training_rays_in_maskcache_sampling(rgb_tr_ori, train_poses, HW, Ks, ndc, inverse_y,
                                            flip_x, flip_y, model, render_kwargs):
    """Rays of all views that hit the coarse geometry, in view and pixel order
    (lib/dvgo.py:582-624): per view the rays, the hit test and an
    order-preserving compaction, all on the device."""
    assert len(rgb_tr_ori) == len(train_poses) == len(Ks) == len(HW)
    N = sum(im.shape[0] * im.shape[1] for im in rgb_tr_ori)
    rgb_tr = torch.zeros([N, 3], device="cuda")
    rays_o_tr = torch.zeros_like(rgb_tr)
    rays_d_tr = torch.zeros_like(rgb_tr)
    viewdirs_tr = torch.zeros_like(rgb_tr)
    imsz, top = [], 0
    for c2w, img, (H, W), K in zip(train_poses, rgb_tr_ori, HW, Ks):
        assert tuple(img.shape[:2]) == (int(H), int(W))
        o, d, v = get_rays_of_a_view(int(H), int(W), K, c2w, ndc, inverse_y, flip_x, flip_y)
        hit = hit_coarse_geo(o, d, render_kwargs["near"], render_kwargs.get("far", 1e9),
                             render_kwargs["stepsize"], xyz_min=model.xyz_min,
                             xyz_max=model.xyz_max, voxel_size=model.voxel_size,
                             mask_cache=model.mask_cache)
        rgb = torch.as_tensor(img).to(device="cuda", dtype=torch.float32).reshape(-1, 3)
        (ro, rd, vd, rc), n = _compact(hit, [o, d, v, rgb], int(H) * int(W))
        rgb_tr[top:top + n].copy_(rc)
        rays_o_tr[top:top + n].copy_(ro)
        rays_d_tr[top:top + n].copy_(rd)
        viewdirs_tr[top:top + n].copy_(vd)
        imsz.append(n)
        top += n
    return rgb_tr[:top], rays_o_tr[:top], rays_d_tr[:top], viewdirs_tr[:top], imsz


def batch_indices_generator(N, BS):
    """Endless batches of a numpy permutation, re-drawn when exhausted
    (lib/dvgo.py:627-634): the same index stream as the reference for the same
    numpy random state."""
    perm, pos = None, 0
    while True:
        if perm is None or pos + BS > N:
            perm, pos = torch.from_numpy(np.random.permutation(N).astype(np.int64)), 0
        yield perm[pos:pos + BS]
        pos += BS
