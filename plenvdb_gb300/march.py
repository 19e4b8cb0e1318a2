"""Fused ray-march stages as torch.autograd.Functions, one per stage:

* ``MarchSample`` (sample): rays -> colour-row weights, alphainv_last and k0
  features. Fuses sample_pts_on_rays, the bbox/mask filter, DensityVDB
  trilinear, Raw2Alpha, Alphas2Weights and ColorVDB trilinear
  (dvgo.py:306-341). Its backward recomputes transmittance from the saved
  per-ray alphas and adds the density and k0 voxel gradients through a
  deterministic leaf-sorted segmented reduction (no float atomics).
* ``RgbNetFn`` (MLP): k0 rows + per-ray view-dir PE -> sigmoid rgb
  (dvgo.py:354-362).
* ``CompositeFn`` (composite): sum over a ray's rows of weight*rgb plus
  alphainv_last*bg (dvgo.py:365-370), deterministic per-ray sums.

The voxel gradients land in the grids' own gradient storage (as the reference's
QueryVerticalInVDB does); the stage Functions take a dummy tensor that
requires grad so autograd runs their backward.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .plenvdb import device_view


def march_params(xyz_min, xyz_max, near, stepdist, act_shift, interval, fast_color_thres,
                 bg=0.0, t_stop=1e-3, far=1e9) -> L.MarchParams:
    p = L.MarchParams()
    for a in range(3):
        p.xyz_min[a] = float(xyz_min[a])
        p.xyz_max[a] = float(xyz_max[a])
    p.near_ = float(near)
    p.far_ = float(far)
    p.stepdist = float(stepdist)
    p.act_shift = float(act_shift)
    p.interval = float(interval)
    p.fast_color_thres = float(fast_color_thres)
    p.t_stop = float(t_stop)
    p.bg = float(bg)
    return p


class MarchWorkspace:
    """Owns a pvdb_march workspace for up to max_rays rays."""

    def __init__(self, max_rays: int, xyz_min, xyz_max, stepdist: float, samples_cap: int = 0,
                 leaf_staging: bool = False):
        lib = L.load()
        if samples_cap <= 0:
            samples_cap = lib.pvdb_march_samples_cap(L.f32arr(xyz_min), L.f32arr(xyz_max),
                                                     float(stepdist))
        self.max_rays = int(max_rays)
        self.samples_cap = int(samples_cap)
        out = C.c_void_p()
        L.call("pvdb_march_create", self.max_rays, self.samples_cap, C.byref(out))
        self.h = out
        self.generation = 0
        self.k0_channels = 0
        self.n_rays = 0
        if leaf_staging:
            self.set_leaf_staging(True)

    def set_leaf_staging(self, on: bool) -> None:
        """Stage the density leaves of the forward's density pass in shared
        memory (bulk copies); bitwise the same results."""
        L.call("pvdb_march_set_leaf_staging", self.h, 1 if on else 0)

    def __del__(self):
        try:
            if self.h:
                L.load().pvdb_march_destroy(self.h)
                self.h = C.c_void_p(None)
        except Exception:
            pass

    def views(self) -> L.MarchViews:
        v = L.MarchViews()
        L.call("pvdb_march_views", self.h, C.byref(v))
        return v

    def totals(self):
        tk, tr = C.c_int64(), C.c_int64()
        L.call("pvdb_march_totals", self.h, C.byref(tk), C.byref(tr), L.stream_of())
        return tk.value, tr.value

    def stats(self):
        """(kept samples, colour rows, samples evaluated) of the last forward."""
        k, r, e = C.c_int64(), C.c_int64(), C.c_int64()
        L.call("pvdb_march_stats", self.h, C.byref(k), C.byref(r), C.byref(e), L.stream_of())
        return k.value, r.value, e.value

    def rows(self, M: int, C0: int):
        """Torch views of the colour rows of the last forward."""
        v = self.views()
        R = self.n_rays
        out = {
            "alphainv_last": device_view(v.alphainv_last, (R,), "float32", self),
            "n_color": device_view(v.n_color, (R,), "int32", self),
            "weight": device_view(v.weight, (M,), "float32", self),
            "alpha": device_view(v.alpha, (M,), "float32", self),
            "ray_id": device_view(v.ray_id, (M,), "int32", self),
            "step_id": device_view(v.step_id, (M,), "int32", self),
        }
        if C0:
            out["k0"] = device_view(v.k0, (M, C0), "float32", self)
        return out


class MarchSample(torch.autograd.Function):
    """Sample stage: (dummy, rays) -> (weight [M], alphainv_last [R], k0 [M,C], ray_id [M])."""

    @staticmethod
    def forward(ctx, dummy, ws: MarchWorkspace, density, k0, rays_o, rays_d, params, mask=None):
        rays_o = rays_o.float().contiguous()
        rays_d = rays_d.float().contiguous()
        R = rays_o.shape[0]
        if R > ws.max_rays:
            raise ValueError(f"{R} rays exceed the workspace capacity {ws.max_rays}")
        mshape = None
        mptr = None
        if mask is not None:
            mask = mask.to(torch.uint8).contiguous()
            mshape = L.i32arr(mask.shape)
            mptr = L.ptr(mask)
        L.call("pvdb_march_forward", ws.h, density.handle, k0.handle if k0 is not None else None,
               L.ptr(rays_o), L.ptr(rays_d), R, C.byref(params), mptr, mshape, L.stream_of())
        ws.n_rays = R
        ws.generation += 1
        C0 = k0.ndim if k0 is not None else 0
        ws.k0_channels = C0
        _, M = ws.totals()
        rows = ws.rows(M, C0)
        ctx.ws, ctx.gen, ctx.density, ctx.k0 = ws, ws.generation, density, k0
        ctx.M, ctx.R, ctx.C0 = M, R, C0
        k0_rows = rows["k0"] if C0 else torch.zeros(M, 0, device=rays_o.device)
        ctx.mark_non_differentiable(rows["ray_id"])
        return rows["weight"], rows["alphainv_last"], k0_rows, rows["ray_id"]

    @staticmethod
    def backward(ctx, g_weight, g_last, g_k0, _g_ray):
        ws = ctx.ws
        if ws.generation != ctx.gen:
            raise RuntimeError("march workspace was reused before this backward ran")
        dev = torch.device("cuda")
        gw = (g_weight if g_weight is not None else torch.zeros(ctx.M, device=dev)).float().contiguous()
        gl = (g_last if g_last is not None else torch.zeros(ctx.R, device=dev)).float().contiguous()
        gk = None
        if ctx.k0 is not None and g_k0 is not None:
            gk = g_k0.float().contiguous()
        L.call("pvdb_march_backward", ws.h, ctx.density.handle,
               ctx.k0.handle if ctx.k0 is not None else None, L.ptr(gw), L.ptr(gl),
               L.ptr(gk) if gk is not None else None, L.stream_of())
        return (None,) * 8


def _mlp_struct(w0, b0, w1, b1, w2, b2, c0, pe) -> L.MlpWeights:
    s = L.MlpWeights()
    s.w0, s.b0, s.w1, s.b1, s.w2, s.b2 = (L.ptr(t) for t in (w0, b0, w1, b1, w2, b2))
    s.c0, s.pe, s.width = int(c0), int(pe), int(w1.shape[0])
    return s


class RgbNetFn(torch.autograd.Function):
    """MLP stage on the rows of the last MarchSample: rgb = sigmoid(rgbnet([k0, PE]))."""

    @staticmethod
    def forward(ctx, k0, viewdirs, ws: MarchWorkspace, pe, precision, w0, b0, w1, b1, w2, b2):
        M = k0.shape[0]
        k0 = k0.detach().float().contiguous()
        viewdirs = viewdirs.float().contiguous()
        ws_params = [t.detach().float().contiguous() for t in (w0, b0, w1, b1, w2, b2)]
        rgb = torch.empty(M, 3, device=k0.device, dtype=torch.float32)
        s = _mlp_struct(*ws_params, k0.shape[1], pe)
        if M:
            L.call("pvdb_mlp_forward", ws.h, C.byref(s), L.ptr(k0), L.ptr(viewdirs), L.ptr(rgb),
                   int(precision), L.stream_of())
        ctx.save_for_backward(k0, viewdirs, rgb, *ws_params)
        ctx.ws, ctx.pe, ctx.precision, ctx.gen = ws, pe, precision, ws.generation
        ctx.c0 = k0.shape[1]
        return rgb

    @staticmethod
    def backward(ctx, g_rgb):
        k0, viewdirs, rgb, w0, b0, w1, b1, w2, b2 = ctx.saved_tensors
        ws = ctx.ws
        if ws.generation != ctx.gen:
            raise RuntimeError("march workspace was reused before this backward ran")
        M = rgb.shape[0]
        grads = [torch.zeros_like(t) for t in (w0, b0, w1, b1, w2, b2)]
        gk0 = torch.zeros(M, ctx.c0, device=rgb.device, dtype=torch.float32)
        if M:
            s = _mlp_struct(w0, b0, w1, b1, w2, b2, ctx.c0, ctx.pe)
            g = L.MlpGrads()
            g.w0, g.b0, g.w1, g.b1, g.w2, g.b2 = (L.ptr(t) for t in grads)
            L.call("pvdb_mlp_backward", ws.h, C.byref(s), L.ptr(k0), L.ptr(viewdirs), L.ptr(rgb),
                   L.ptr(g_rgb.float().contiguous()), C.byref(g), L.ptr(gk0), int(ctx.precision),
                   L.stream_of())
        return (gk0, None, None, None, None, *grads)


class CompositeFn(torch.autograd.Function):
    """Composite stage: rgb_marched[r] = sum_rows weight*rgb + alphainv_last*bg."""

    @staticmethod
    def forward(ctx, weight, rgb, alphainv_last, ws: MarchWorkspace, bg):
        R = alphainv_last.shape[0]
        rgb = rgb.float().contiguous()
        out = torch.empty(R, 3, device=rgb.device, dtype=torch.float32)
        L.call("pvdb_composite_forward", ws.h, L.ptr(rgb), float(bg), L.ptr(out), R,
               L.stream_of())
        ctx.save_for_backward(rgb)
        ctx.ws, ctx.bg, ctx.R, ctx.gen = ws, float(bg), R, ws.generation
        return out

    @staticmethod
    def backward(ctx, g):
        (rgb,) = ctx.saved_tensors
        ws = ctx.ws
        if ws.generation != ctx.gen:
            raise RuntimeError("march workspace was reused before this backward ran")
        M = rgb.shape[0]
        g = g.float().contiguous()
        grad_rgb = torch.empty(M, 3, device=rgb.device, dtype=torch.float32)
        grad_w = torch.empty(M, device=rgb.device, dtype=torch.float32)
        grad_last = torch.zeros(ctx.R, device=rgb.device, dtype=torch.float32)
        L.call("pvdb_composite_backward", ws.h, L.ptr(rgb), L.ptr(g), ctx.bg, L.ptr(grad_rgb),
               L.ptr(grad_w), L.ptr(grad_last), ctx.R, L.stream_of())
        return grad_w, grad_rgb, grad_last, None, None
