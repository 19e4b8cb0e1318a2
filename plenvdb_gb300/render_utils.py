"""render_utils_cuda for the standalone (unfused) DirectVoxGO path: the same
function names, argument order and return tuples as the reference's torch
extension (lib/cuda/render_utils.cpp:170-184), on CUDA tensors, backed by
libpvdb's kernels (pvdb_ray_*, pvdb_maskcache_lookup, pvdb_raw2alpha*,
pvdb_alpha2weight*). The calls run on the current torch stream and do not
synchronise, except sample_pts_on_rays, which reads the total sample count
back (as the reference does, render_utils_kernel.cu:212)."""
from __future__ import annotations

import torch

from . import _lib as L


def _f32(t):
    return t.detach().float().contiguous()


def _vec3(t):
    v = t.detach().float().cpu().reshape(-1).tolist() if torch.is_tensor(t) else list(t)
    return L.f32arr([float(x) for x in v])


def infer_t_minmax(rays_o, rays_d, xyz_min, xyz_max, near, far):
    """(t_min, t_max) per ray (render_utils_kernel.cu:12-32)."""
    t_min, t_max, _ = _count(rays_o, rays_d, xyz_min, xyz_max, near, far, 1.0)
    return t_min, t_max


def _count(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist):
    ro, rd = _f32(rays_o), _f32(rays_d)
    R = ro.shape[0]
    t_min = torch.empty(R, device=ro.device, dtype=torch.float32)
    t_max = torch.empty_like(t_min)
    n = torch.empty(R, device=ro.device, dtype=torch.int64)
    L.call("pvdb_ray_count_samples", L.ptr(ro), L.ptr(rd), R, _vec3(xyz_min), _vec3(xyz_max),
           float(near), float(far), float(stepdist), L.ptr(t_min), L.ptr(t_max), L.ptr(n),
           L.stream_of())
    return t_min, t_max, n


def sample_pts_on_rays(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist):
    """(ray_pts, mask_outbbox, ray_id, step_id, N_steps, t_min, t_max)
    (render_utils_kernel.cu:196-242)."""
    ro, rd = _f32(rays_o), _f32(rays_d)
    t_min, t_max, n_steps = _count(ro, rd, xyz_min, xyz_max, near, far, stepdist)
    csum = torch.cumsum(n_steps, 0)
    total = int(csum[-1].item()) if csum.numel() else 0
    dev = ro.device
    pts = torch.empty(total, 3, device=dev, dtype=torch.float32)
    ob = torch.empty(total, device=dev, dtype=torch.bool)
    rid = torch.empty(total, device=dev, dtype=torch.int64)
    sid = torch.empty(total, device=dev, dtype=torch.int64)
    if total:
        L.call("pvdb_ray_sample_points", L.ptr(ro), L.ptr(rd), ro.shape[0], _vec3(xyz_min),
               _vec3(xyz_max), float(stepdist), L.ptr(t_min), L.ptr(csum), total, L.ptr(pts),
               L.ptr(ob), L.ptr(rid), L.ptr(sid), L.stream_of())
    return pts, ob, rid, sid, n_steps, t_min, t_max


def maskcache_lookup(world, xyz, xyz2ijk_scale, xyz2ijk_shift):
    """world[round(xyz * scale + shift)], False outside (render_utils_kernel.cu:373-424)."""
    w = world.detach().to(torch.uint8).contiguous()
    x = _f32(xyz)
    out = torch.empty(x.shape[0], device=x.device, dtype=torch.bool)
    if x.shape[0]:
        L.call("pvdb_maskcache_lookup", L.ptr(w), L.i32arr(list(w.shape)), L.ptr(x), x.shape[0],
               _vec3(xyz2ijk_scale), _vec3(xyz2ijk_shift), L.ptr(out), L.stream_of())
    return out


def raw2alpha(density, shift, interval):
    """(exp, alpha) (render_utils_kernel.cu:430-443)."""
    d = _f32(density)
    e = torch.empty_like(d)
    a = torch.empty_like(d)
    if d.numel():
        L.call("pvdb_raw2alpha", L.ptr(d), d.numel(), float(shift), float(interval), L.ptr(e),
               L.ptr(a), L.stream_of())
    return e, a


def raw2alpha_backward(exp, grad_back, interval):
    """d alpha / d density * grad_back (render_utils_kernel.cu:506-517)."""
    e, g = _f32(exp), _f32(grad_back)
    out = torch.empty_like(e)
    if e.numel():
        L.call("pvdb_raw2alpha_backward", L.ptr(e), L.ptr(g), e.numel(), float(interval),
               L.ptr(out), L.stream_of())
    return out


def alpha2weight(alpha, ray_id, n_rays):
    """(weights, T, alphainv_last, i_start, i_end) for points sorted by ray
    (render_utils_kernel.cu:576-651)."""
    a = _f32(alpha)
    rid = ray_id.detach().to(torch.int64).contiguous()
    n = a.numel()
    dev = a.device
    w = torch.empty_like(a)
    T = torch.empty_like(a)
    last = torch.empty(n_rays, device=dev, dtype=torch.float32)
    i_s = torch.empty(n_rays, device=dev, dtype=torch.int64)
    i_e = torch.empty(n_rays, device=dev, dtype=torch.int64)
    L.call("pvdb_alpha2weight", L.ptr(a), L.ptr(rid), n, int(n_rays), L.ptr(w), L.ptr(T),
           L.ptr(last), L.ptr(i_s), L.ptr(i_e), L.stream_of())
    return w, T, last, i_s, i_e


def alpha2weight_backward(alpha, weight, T, alphainv_last, i_start, i_end, n_rays,
                          grad_weights, grad_last):
    """Gradient w.r.t. alpha (render_utils_kernel.cu:653-707)."""
    a = _f32(alpha)
    out = torch.empty_like(a)
    L.call("pvdb_alpha2weight_backward", L.ptr(a), L.ptr(_f32(weight)), L.ptr(_f32(T)),
           L.ptr(_f32(alphainv_last)), L.ptr(i_start.contiguous()), L.ptr(i_end.contiguous()),
           int(n_rays), L.ptr(_f32(grad_weights)), L.ptr(_f32(grad_last)), a.numel(),
           L.ptr(out), L.stream_of())
    return out
