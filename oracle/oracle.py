"""ORACLE — test infrastructure only (tests/, the smoke check, bench.py's CPU
baseline). Python wrapper of the CPU restatement in pvdb_oracle.cpp.

Grids are described by `OGridData`: resolution, dense values over [0,reso)^3
(padded here to whole leaves), the active mask, which leaves are allocated
(default: the leaves holding an active voxel) and the background.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build_oracle()
        _lib = C.CDLL(path)
        _lib.oracle_march_run.restype = C.c_void_p
        _lib.oracle_march_rows.restype = C.c_int64
        _lib.oracle_march_kept.restype = C.c_int64
        for n in ("oracle_march_rows", "oracle_march_kept", "oracle_march_free"):
            getattr(_lib, n).argtypes = [C.c_void_p]
    return _lib


class _OGrid(C.Structure):
    _fields_ = [("reso", C.c_int * 3), ("pad", C.c_int * 3), ("C", C.c_int),
                ("background", C.c_float), ("alloc", C.c_void_p), ("active", C.c_void_p),
                ("values", C.c_void_p)]


class _MarchParams(C.Structure):
    _fields_ = [("xyz_min", C.c_float * 3), ("xyz_max", C.c_float * 3), ("near_", C.c_float),
                ("far_", C.c_float), ("stepdist", C.c_float), ("act_shift", C.c_float),
                ("interval", C.c_float), ("fast_color_thres", C.c_float), ("t_stop", C.c_float),
                ("bg", C.c_float)]


class _Mlp(C.Structure):
    _fields_ = [("w0", C.c_void_p), ("b0", C.c_void_p), ("w1", C.c_void_p), ("b1", C.c_void_p),
                ("w2", C.c_void_p), ("b2", C.c_void_p), ("c0", C.c_int), ("pe", C.c_int),
                ("width", C.c_int)]


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


@dataclass
class OGridData:
    reso: tuple
    values: np.ndarray        # [R0,R1,R2,C] (or [R0,R1,R2] for C == 1)
    active: np.ndarray        # [R0,R1,R2] bool/uint8
    background: float = 0.0
    alloc: np.ndarray | None = None  # [L0,L1,L2] uint8; None = leaves holding an active voxel
    inactive_value: float | None = None  # value stored at inactive in-leaf voxels (None: keep)

    def __post_init__(self):
        R = [int(r) for r in self.reso]
        self.reso = tuple(R)
        self.pad = tuple(8 * ((r + 7) // 8) for r in R)
        v = np.asarray(self.values, np.float64)
        if v.ndim == 3:
            v = v[..., None]
        self.C = v.shape[-1]
        act = np.asarray(self.active).astype(np.uint8)
        P = self.pad
        self.p_active = np.zeros(P, np.uint8)
        a0, a1, a2 = act.shape
        self.p_active[:a0, :a1, :a2] = act
        self.p_active[R[0]:, :, :] = 0
        self.p_active[:, R[1]:, :] = 0
        self.p_active[:, :, R[2]:] = 0
        fill = self.background if self.inactive_value is None else self.inactive_value
        self.p_values = np.full(P + (self.C,), fill, np.float64)
        # values may cover [0,reso) or the whole padded leaf box
        v0, v1, v2 = v.shape[:3]
        self.p_values[:v0, :v1, :v2] = v
        if self.inactive_value is not None:
            self.p_values[self.p_active == 0] = self.inactive_value
        if self.alloc is None:
            L = [p // 8 for p in P]
            self.alloc = self.p_active.reshape(L[0], 8, L[1], 8, L[2], 8).max(axis=(1, 3, 5))
        self.alloc = np.ascontiguousarray(np.asarray(self.alloc, np.uint8))
        self.p_values = np.ascontiguousarray(self.p_values.reshape(-1))
        self.p_active = np.ascontiguousarray(self.p_active)
        self._s = _OGrid()
        self._s.reso[:] = list(self.reso)
        self._s.pad[:] = list(self.pad)
        self._s.C = self.C
        self._s.background = self.background
        self._s.alloc = self.alloc.ctypes.data
        self._s.active = self.p_active.ctypes.data
        self._s.values = self.p_values.ctypes.data

    @property
    def ref(self):
        return C.byref(self._s)

    def dense(self, which_values=None) -> np.ndarray:
        """Values over [0,reso) as the grid reads them (background outside leaves)."""
        R, P = self.reso, self.pad
        v = (self.p_values if which_values is None else which_values).reshape(P + (self.C,))
        L = [p // 8 for p in P]
        allocv = np.repeat(np.repeat(np.repeat(self.alloc, 8, 0), 8, 1), 8, 2).astype(bool)
        out = np.where(allocv[..., None], v, self.background)
        return out[:R[0], :R[1], :R[2]]

    def padded_zeros(self) -> np.ndarray:
        return np.zeros(int(np.prod(self.pad)) * self.C, np.float64)

    def unpad(self, arr: np.ndarray) -> np.ndarray:
        R = self.reso
        return arr.reshape(self.pad + (self.C,))[:R[0], :R[1], :R[2]]


def lookup(g: OGridData, ijk: np.ndarray):
    ijk = np.ascontiguousarray(ijk, np.int32)
    n = ijk.shape[0]
    out = np.empty(n * g.C)
    act = np.empty(n, np.uint8)
    lib().oracle_lookup(g.ref, _p(ijk), C.c_int64(n), _p(out), _p(act))
    return out.reshape(n, g.C), act


def sample(g: OGridData, xyz: np.ndarray, fp32: bool = False):
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = xyz.shape[0]
    out = np.empty(n * g.C)
    lib().oracle_sample(g.ref, _p(xyz), C.c_int64(n), int(fp32), _p(out))
    return out.reshape(n, g.C)


def sample_backward(g: OGridData, xyz: np.ndarray, grad: np.ndarray):
    xyz = np.ascontiguousarray(xyz, np.float32)
    grad = np.ascontiguousarray(grad, np.float64).reshape(-1)
    out = g.padded_zeros()
    lib().oracle_sample_backward(g.ref, _p(xyz), _p(grad), C.c_int64(xyz.shape[0]), _p(out))
    return g.unpad(out)


def adam(g: OGridData, grad_pad, m_pad, v_pad, perlr_pad, stepsz, eps, b0, b1, mode, fp32=False):
    """One voxel-Adam step on padded arrays (modified in place); returns data."""
    data = g.p_values.copy()
    lib().oracle_adam(g.ref, _p(data), _p(grad_pad), _p(m_pad), _p(v_pad), _p(perlr_pad),
                      C.c_float(stepsz), C.c_float(eps), C.c_float(b0), C.c_float(b1), int(mode),
                      int(fp32))
    return data


def tv(g: OGridData, grad_pad, wx, wy, wz, dense_mode, fp32=False):
    """TV gradient with weights already divided by 6, added into grad_pad
    (fp32: the reference's float arithmetic)."""
    lib().oracle_tv(g.ref, _p(grad_pad), C.c_float(wx), C.c_float(wy), C.c_float(wz),
                    int(dense_mode), int(fp32))
    return grad_pad


def adam_step_size(lr, beta1, beta2, step):
    """Host-side Adam step size of adam_upd_kernel.cu:72 (float)."""
    f = lib().oracle_adam_step_size
    f.restype = C.c_float
    return float(f(C.c_float(lr), C.c_float(beta1), C.c_float(beta2), int(step)))


def adam_dense(p, g, m, v, perlr, step, beta1, beta2, lr, eps, mode, fp32=False):
    """One dense Adam step (MaskedAdam's kernels) on float64 copies; returns
    (p, m, v)."""
    p, m, v = (np.array(x, np.float64) for x in (p, m, v))
    g = np.ascontiguousarray(g, np.float64)
    pl = None if perlr is None else np.ascontiguousarray(perlr, np.float64)
    lib().oracle_adam_dense(_p(p), _p(g), _p(m), _p(v), _p(pl), C.c_int64(p.size), int(step),
                            C.c_float(beta1), C.c_float(beta2), C.c_float(lr), C.c_float(eps),
                            int(mode), int(fp32))
    return p, m, v


def raw2alpha(d, shift, interval, fp32=False):
    d = np.ascontiguousarray(d, np.float32)
    e, a = np.empty(d.size), np.empty(d.size)
    lib().oracle_raw2alpha(_p(d), C.c_int64(d.size), C.c_float(shift), C.c_float(interval),
                           int(fp32), _p(e), _p(a))
    return e, a


def raw2alpha_backward(e, g, interval, fp32=False):
    e = np.ascontiguousarray(e, np.float64)
    g = np.ascontiguousarray(g, np.float64)
    out = np.empty(e.size)
    lib().oracle_raw2alpha_backward(_p(e), _p(g), C.c_int64(e.size), C.c_float(interval),
                                    int(fp32), _p(out))
    return out


def alpha2weight(alpha, ray_id, n_rays, fp32=False):
    alpha = np.ascontiguousarray(alpha, np.float64)
    ray_id = np.ascontiguousarray(ray_id, np.int64)
    n = alpha.size
    w, T = np.empty(n), np.empty(n)
    last = np.empty(n_rays)
    i_s, i_e = np.empty(n_rays, np.int64), np.empty(n_rays, np.int64)
    lib().oracle_alpha2weight(_p(alpha), _p(ray_id), C.c_int64(n), int(n_rays), int(fp32), _p(w),
                              _p(T), _p(last), _p(i_s), _p(i_e))
    return w, T, last, i_s, i_e


def alpha2weight_backward(alpha, w, T, last, i_s, i_e, gw, gl, fp32=False):
    n = len(alpha)
    out = np.empty(n)
    arrs = [np.ascontiguousarray(x, np.float64) for x in (alpha, w, T, last, gw, gl)]
    i_s = np.ascontiguousarray(i_s, np.int64)
    i_e = np.ascontiguousarray(i_e, np.int64)
    lib().oracle_alpha2weight_backward(_p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
                                       _p(i_s), _p(i_e), int(len(last)), _p(arrs[4]), _p(arrs[5]),
                                       C.c_int64(n), int(fp32), _p(out))
    return out


def march_params(xyz_min, xyz_max, near, stepdist, act_shift, interval, thres, bg=0.0,
                 t_stop=1e-3, far=1e9):
    p = _MarchParams()
    p.xyz_min[:] = [float(x) for x in xyz_min]
    p.xyz_max[:] = [float(x) for x in xyz_max]
    p.near_, p.far_, p.stepdist = near, far, stepdist
    p.act_shift, p.interval, p.fast_color_thres = act_shift, interval, thres
    p.t_stop, p.bg = t_stop, bg
    return p


def ray_count(rays_o, rays_d, p):
    ro = np.ascontiguousarray(rays_o, np.float32)
    rd = np.ascontiguousarray(rays_d, np.float32)
    R = ro.shape[0]
    tmin, tmax = np.empty(R, np.float32), np.empty(R, np.float32)
    ns = np.empty(R, np.int64)
    lib().oracle_ray_count(_p(ro), _p(rd), int(R), C.byref(p), _p(tmin), _p(tmax), _p(ns))
    return tmin, tmax, ns


def ray_points(rays_o, rays_d, p):
    ro = np.ascontiguousarray(rays_o, np.float32)
    rd = np.ascontiguousarray(rays_d, np.float32)
    _, _, ns = ray_count(ro, rd, p)
    tot = int(ns.sum())
    pts = np.empty((tot, 3), np.float32)
    ob = np.empty(tot, np.uint8)
    rid, sid = np.empty(tot, np.int64), np.empty(tot, np.int64)
    lib().oracle_ray_points(_p(ro), _p(rd), int(ro.shape[0]), C.byref(p), _p(pts), _p(ob),
                            _p(rid), _p(sid))
    return pts, ob.astype(bool), rid, sid


def maskcache(world, xyz, scale, shift):
    world = np.ascontiguousarray(world, np.uint8)
    xyz = np.ascontiguousarray(xyz, np.float32)
    sh = np.ascontiguousarray(np.array(world.shape, np.int32))
    sc = np.ascontiguousarray(scale, np.float32)
    sf = np.ascontiguousarray(shift, np.float32)
    out = np.empty(xyz.shape[0], np.uint8)
    lib().oracle_maskcache(_p(world), _p(sh), _p(xyz), C.c_int64(xyz.shape[0]), _p(sc), _p(sf),
                           _p(out))
    return out.astype(bool)


class MLPWeights:
    """rgbnet weights in nn.Linear layout, float64."""

    def __init__(self, w0, b0, w1, b1, w2, b2, c0, pe):
        self.arrs = [np.ascontiguousarray(np.asarray(x, np.float64)) for x in (w0, b0, w1, b1, w2, b2)]
        self.c0, self.pe, self.width = int(c0), int(pe), int(self.arrs[2].shape[0])
        self._s = _Mlp()
        self._s.w0, self._s.b0, self._s.w1, self._s.b1, self._s.w2, self._s.b2 = (
            a.ctypes.data for a in self.arrs)
        self._s.c0, self._s.pe, self._s.width = self.c0, self.pe, self.width

    @property
    def ref(self):
        return C.byref(self._s)


class March:
    """DirectVoxGO forward (dvgo.py:296-370) on the oracle; fp32 mimics the reference."""

    def __init__(self, gd: OGridData, gk: OGridData | None, rays_o, rays_d, params, fp32=False):
        self.gd, self.gk, self.params = gd, gk, params
        self.ro = np.ascontiguousarray(rays_o, np.float32)
        self.rd = np.ascontiguousarray(rays_d, np.float32)
        self.R = self.ro.shape[0]
        self.fp32 = fp32
        self.h = C.c_void_p(lib().oracle_march_run(gd.ref, gk.ref if gk else None, _p(self.ro),
                                                   _p(self.rd), int(self.R), C.byref(params),
                                                   int(fp32)))
        self.M = int(lib().oracle_march_rows(self.h))
        self.K = int(lib().oracle_march_kept(self.h))
        Cc = gk.C if gk else 0
        self.T_last = np.empty(self.R)
        self.n_kept = np.empty(self.R, np.int32)
        self.n_color = np.empty(self.R, np.int32)
        self.k0 = np.empty((self.M, Cc))
        self.weight = np.empty(self.M)
        self.alpha = np.empty(self.M)
        self.ray_id = np.empty(self.M, np.int32)
        self.step_id = np.empty(self.M, np.int32)
        self.kept_alpha = np.empty(self.K)
        self.kept_step = np.empty(self.K, np.int32)
        lib().oracle_march_fetch(self.h, _p(self.T_last), _p(self.n_kept), _p(self.n_color),
                                 _p(self.k0), _p(self.weight), _p(self.alpha), _p(self.ray_id),
                                 _p(self.step_id), _p(self.kept_alpha), _p(self.kept_step))

    def __del__(self):
        try:
            lib().oracle_march_free(self.h)
        except Exception:
            pass

    def rgb(self, mlp: MLPWeights, viewdirs):
        vd = np.ascontiguousarray(viewdirs, np.float32)
        out = np.empty((self.M, 3))
        lib().oracle_march_rgb(self.h, mlp.ref, _p(vd), _p(out))
        return out

    def composite(self, rgb, bg):
        out = np.zeros((self.R, 3))
        np.add.at(out, self.ray_id, self.weight[:, None] * rgb)
        return out + self.T_last[:, None] * bg

    def backward_sample(self, g_w, g_last, g_k0=None):
        """FP64 sample-stage gradients: (density [R^3], k0 [R^3,C] or None)."""
        assert not self.fp32
        gd_pad = self.gd.padded_zeros()
        gk_pad = self.gk.padded_zeros() if self.gk is not None else None
        gw = np.ascontiguousarray(g_w, np.float64)
        gl = np.ascontiguousarray(g_last, np.float64)
        gk = None if g_k0 is None else np.ascontiguousarray(g_k0, np.float64).reshape(-1)
        lib().oracle_march_backward_sample(self.h, self.gd.ref,
                                           self.gk.ref if self.gk is not None else None,
                                           C.byref(self.params), _p(gw), _p(gl), _p(gk),
                                           _p(gd_pad), _p(gk_pad))
        return (self.gd.unpad(gd_pad)[..., 0],
                self.gk.unpad(gk_pad) if gk_pad is not None else None)

    def backward(self, mlp: MLPWeights, viewdirs, g_rgbm, g_last=None, g_rgb=None):
        """FP64 gradients: (density [R^3], k0 [R^3,C], [gw0,gb0,gw1,gb1,gw2,gb2])."""
        assert not self.fp32
        vd = np.ascontiguousarray(viewdirs, np.float32)
        gd_pad = self.gd.padded_zeros()
        gk_pad = self.gk.padded_zeros()
        grads = [np.zeros_like(a) for a in mlp.arrs]
        g_rgbm = np.ascontiguousarray(g_rgbm, np.float64)
        gl = None if g_last is None else np.ascontiguousarray(g_last, np.float64)
        gr = None if g_rgb is None else np.ascontiguousarray(g_rgb, np.float64)
        lib().oracle_march_backward(self.h, self.gd.ref, self.gk.ref, mlp.ref, _p(vd),
                                    C.byref(self.params), _p(g_rgbm), _p(gl), _p(gr), _p(gd_pad),
                                    _p(gk_pad), *[_p(g) for g in grads])
        return self.gd.unpad(gd_pad)[..., 0], self.gk.unpad(gk_pad), grads


class _TrainGrids(C.Structure):
    _fields_ = [("reso", C.c_int * 3), ("pad", C.c_int * 3), ("background", C.c_float),
                ("alloc", C.c_void_p), ("active", C.c_void_p), ("dens", C.c_void_p),
                ("k0", C.c_void_p), ("gdens", C.c_void_p), ("gk0", C.c_void_p),
                ("m_d", C.c_void_p), ("v_d", C.c_void_p), ("m_k", C.c_void_p),
                ("v_k", C.c_void_p), ("C", C.c_int), ("step", C.c_int), ("lr_d", C.c_float),
                ("lr_k", C.c_float)]


class _TrainNet(C.Structure):
    _fields_ = [("params", C.c_void_p), ("grads", C.c_void_p), ("m", C.c_void_p),
                ("v", C.c_void_p), ("c0", C.c_int), ("pe", C.c_int), ("width", C.c_int),
                ("step", C.c_int), ("lr", C.c_float)]


class CPUTrainer:
    """The fine-stage iteration in FP32 on the host cores (oracle_train_step_fp32):
    the CPU implementation of the path used as the reported baseline."""

    def __init__(self, reso, density, k0, active, background, rgbnet_params, lr_d=0.1,
                 lr_k=0.075, lr_net=1e-3):
        R = [int(r) for r in reso]
        P = [8 * ((r + 7) // 8) for r in R]
        self.act = np.zeros(P, np.uint8)
        self.act[:R[0], :R[1], :R[2]] = active
        L = [p // 8 for p in P]
        self.alloc = np.ascontiguousarray(self.act.reshape(L[0], 8, L[1], 8, L[2], 8).max(axis=(1, 3, 5)))
        C_ = k0.shape[-1]
        self.dens = np.full(P, background, np.float32)
        self.dens[:R[0], :R[1], :R[2]] = density
        self.k0 = np.zeros(P + [C_], np.float32)
        self.k0[:R[0], :R[1], :R[2]] = k0
        self.gd = np.zeros(P, np.float32)
        self.gk = np.zeros(P + [C_], np.float32)
        self.md, self.vd = np.zeros(P, np.float32), np.zeros(P, np.float32)
        self.mk, self.vk = np.zeros(P + [C_], np.float32), np.zeros(P + [C_], np.float32)
        self.g = _TrainGrids()
        self.g.reso[:] = R
        self.g.pad[:] = P
        self.g.background = background
        for name in ("alloc", "dens", "k0", "gd", "gk", "md", "vd", "mk", "vk"):
            pass
        self.g.alloc, self.g.active = self.alloc.ctypes.data, self.act.ctypes.data
        self.g.dens, self.g.k0 = self.dens.ctypes.data, self.k0.ctypes.data
        self.g.gdens, self.g.gk0 = self.gd.ctypes.data, self.gk.ctypes.data
        self.g.m_d, self.g.v_d = self.md.ctypes.data, self.vd.ctypes.data
        self.g.m_k, self.g.v_k = self.mk.ctypes.data, self.vk.ctypes.data
        self.g.C, self.g.step, self.g.lr_d, self.g.lr_k = C_, 0, lr_d, lr_k
        w0 = np.asarray(rgbnet_params[0])
        self.params = np.ascontiguousarray(np.concatenate(
            [np.asarray(t, np.float32).reshape(-1) for t in rgbnet_params]))
        self.grads = np.zeros_like(self.params)
        self.m, self.v = np.zeros_like(self.params), np.zeros_like(self.params)
        self.n = _TrainNet()
        self.n.params, self.n.grads = self.params.ctypes.data, self.grads.ctypes.data
        self.n.m, self.n.v = self.m.ctypes.data, self.v.ctypes.data
        self.n.c0 = C_
        self.n.pe = (w0.shape[1] - C_ - 3) // 6
        self.n.width = w0.shape[0]
        self.n.step, self.n.lr = 0, lr_net
        lib().oracle_train_step_fp32.restype = C.c_double

    def step(self, rays_o, rays_d, viewdirs, target, params, w_main=1.0, w_ent=1e-3, w_per=1e-2,
             tv_weight=1e-4):
        ro, rd, vd, tg = (np.ascontiguousarray(a, np.float32) for a in (rays_o, rays_d, viewdirs, target))
        R = ro.shape[0]
        tv_w = tv_weight / R * max(self.g.reso) / 128.0 / 6.0 if tv_weight > 0 else 0.0
        return lib().oracle_train_step_fp32(C.byref(self.g), C.byref(self.n), _p(ro), _p(rd), _p(vd),
                                            _p(tg), int(R), C.byref(params), C.c_float(w_main),
                                            C.c_float(w_ent), C.c_float(w_per), C.c_float(tv_w))


    def density_step(self, rays_o, rays_d, target_alpha, params):
        """Density-only FP32 forward + backward with the alpha-MSE loss
        (oracle_density_step_fp32); the gradient accumulates into self.gd."""
        ro, rd, ta = (np.ascontiguousarray(a, np.float32) for a in (rays_o, rays_d, target_alpha))
        f = lib().oracle_density_step_fp32
        f.restype = C.c_double
        return f(C.byref(self.g), _p(ro), _p(rd), _p(ta), int(ro.shape[0]), C.byref(params))


class _RenderParams(C.Structure):
    _fields_ = [("H", C.c_int), ("W", C.c_int), ("inverse_y", C.c_int), ("reso", C.c_int * 3),
                ("K", C.c_float * 9), ("c2w", C.c_float * 16), ("xyz_min", C.c_float * 3),
                ("xyz_max", C.c_float * 3), ("near_", C.c_float), ("stepdist", C.c_float),
                ("shift", C.c_float), ("interval", C.c_float), ("thr", C.c_float),
                ("bg", C.c_float), ("t_stop", C.c_float)]


def render_pixels(index, den, col, mlp: MLPWeights, K, c2w, xyz_min, xyz_max, H, W, near,
                  stepdist, act_shift, interval, thres, bg, t_stop, pixels=None, inverse_y=False,
                  fp32=False):
    """MGRenderer render march (renderer.cu:122-412) for the given pixel ids
    (default: all H*W). index: dense int row ids [R0,R1,R2] (0 = empty);
    den [N]; col [N, dcol]. Returns (rgb [n,3], colour samples [n], T [n])."""
    idx = np.ascontiguousarray(index, np.int32)
    den = np.ascontiguousarray(den, np.float32).reshape(-1)
    col = np.ascontiguousarray(col, np.float32)
    dcol = col.shape[1]
    col = col.reshape(-1)
    pix = np.arange(H * W, dtype=np.int64) if pixels is None else np.ascontiguousarray(pixels, np.int64)
    P = _RenderParams()
    P.H, P.W, P.inverse_y = int(H), int(W), int(bool(inverse_y))
    P.reso[:] = [int(r) for r in idx.shape]
    P.K[:] = [float(v) for v in np.asarray(K, np.float32).reshape(-1)]
    P.c2w[:] = [float(v) for v in np.asarray(c2w, np.float32).reshape(-1)]
    P.xyz_min[:] = [float(v) for v in xyz_min]
    P.xyz_max[:] = [float(v) for v in xyz_max]
    P.near_, P.stepdist, P.shift, P.interval = near, stepdist, act_shift, interval
    P.thr, P.bg, P.t_stop = thres, bg, t_stop
    n = pix.shape[0]
    rgb = np.empty((n, 3))
    ncol = np.empty(n, np.int32)
    T = np.empty(n)
    lib().oracle_render_pixels(C.byref(P), _p(idx), _p(den), _p(col), int(dcol), mlp.ref, _p(pix),
                               C.c_int64(n), int(fp32), _p(rgb), _p(ncol), _p(T))
    return rgb, ncol, T


def index_density(index, den, xyz, fp32=False):
    """Index-grid trilinear density (renderer.cu:271-300) and isActive(Round(xyz))
    at index-space points xyz [n,3]; index: dense row ids [R0,R1,R2]."""
    idx = np.ascontiguousarray(index, np.int32)
    den = np.ascontiguousarray(den, np.float32).reshape(-1)
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = xyz.shape[0]
    reso = np.asarray(idx.shape, np.int32)
    out = np.empty(n)
    act = np.empty(n, np.uint8)
    lib().oracle_index_density(_p(reso), _p(idx), _p(den), _p(xyz), C.c_int64(n), int(fp32),
                               _p(out), _p(act))
    return out, act.astype(bool)


def set_threads(n: int):
    lib().oracle_set_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())
