"""Drop-in replacement of the reference's pybind11 module ``plenvdb``
(plenvdb/lib/vdb/plenvdb.cpp:3-172): classes DensityVDB, ColorVDB, DensityOpt,
ColorOpt and MGRenderer with the same method names and argument meanings.

Arrays may be numpy arrays (host: copied in and out, the call returns a numpy
array, as the reference does) or CUDA torch tensors (device: used in place, the
call returns a CUDA tensor and does not synchronise). Unlike the reference,
dtypes and sizes are checked; a mismatch raises ValueError.

Files written by save_to / load_from use this library's leaf format (topology,
active masks, values and a checksum) under the reference's file names; OpenVDB
.vdb files are not read or written.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _lib as L


def _as_host_f32(x) -> np.ndarray:
    if isinstance(x, np.ndarray):
        a = x
    else:  # torch CPU tensor or sequence
        a = np.asarray(x.detach().cpu().numpy() if hasattr(x, "detach") else x)
    if a.dtype != np.float32:
        a = a.astype(np.float32)
    return np.ascontiguousarray(a)


def _as_host_i32(x) -> np.ndarray:
    a = x if isinstance(x, np.ndarray) else np.asarray(
        x.detach().cpu().numpy() if hasattr(x, "detach") else x)
    return np.ascontiguousarray(a.astype(np.int32, copy=False))


def _as_host_u8(x) -> np.ndarray:
    a = x if isinstance(x, np.ndarray) else np.asarray(
        x.detach().cpu().numpy() if hasattr(x, "detach") else x)
    return np.ascontiguousarray(a.astype(np.uint8, copy=False))


def _dev_f32(t):
    import torch
    if t.dtype != torch.float32:
        t = t.float()
    return t.contiguous()


class _CudaArray:
    """Minimal __cuda_array_interface__ holder to view library memory in torch."""

    def __init__(self, ptr: int, shape, typestr: str, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}
        self._owner = owner


def device_view(ptr: int, shape, dtype: str, owner):
    """Zero-copy torch view of device memory owned by `owner` (kept alive)."""
    import torch
    typestr = {"float32": "<f4", "int32": "<i4", "uint64": "<u8", "uint8": "|u1"}[dtype]
    t = torch.as_tensor(_CudaArray(ptr, shape, typestr, owner), device="cuda")
    return t


class _GridHandle:
    """Owns one pvdb_grid (values + gradient of one channel set)."""

    def __init__(self, handle: int):
        self.h = C.c_void_p(handle)

    def __del__(self):
        try:
            if self.h:
                L.load().pvdb_grid_destroy(self.h)
                self.h = C.c_void_p(None)
        except Exception:
            pass


def _grid_info(h):
    reso = (C.c_int32 * 3)()
    ch, nleaf = C.c_int32(), C.c_int32()
    nact = C.c_int64()
    bg = C.c_float()
    L.call("pvdb_grid_get_info", h, reso, C.byref(ch), C.byref(nleaf), C.byref(nact), C.byref(bg))
    return list(reso), ch.value, nleaf.value, nact.value, bg.value


def _device_arrays(h, owner):
    """Zero-copy torch views of a grid handle's device arrays."""
    d, g, m, t, o = (C.c_void_p() for _ in range(5))
    ld = (C.c_int32 * 3)()
    L.call("pvdb_grid_device_views", h, C.byref(d), C.byref(g), C.byref(m), C.byref(t),
           C.byref(o), ld)
    _, ch, nleaf, _, _ = _grid_info(h)
    return {"data": device_view(d.value, (nleaf * 512 * ch,), "float32", owner),
            "mask": device_view(m.value, (nleaf * 8,), "uint64", owner),
            "table": device_view(t.value, (ld[0] * ld[1] * ld[2],), "int32", owner),
            "origin": device_view(o.value, (nleaf * 3,), "int32", owner)}


def _same_topology(h0, h1) -> bool:
    import torch
    r0, c0, n0, _, _ = _grid_info(h0)
    r1, c1, n1, _, _ = _grid_info(h1)
    if (r0, c0, n0) != (r1, c1, n1):
        return False
    a, b = _device_arrays(h0, None), _device_arrays(h1, None)
    return (torch.equal(a["mask"].view(torch.int64), b["mask"].view(torch.int64))
            and all(torch.equal(a[k], b[k]) for k in ("table", "origin")))


class BaseVDB:
    """Common part of DensityVDB / ColorVDB (plenvdb.h:389-429)."""

    def __init__(self, resolution, n: int, *, _handle: int | None = None,
                 background: float = 0.0):
        n = int(n)
        if n != 1 and (n <= 0 or n % 3):
            raise ValueError("channels must be 1 or a positive multiple of 3")
        self.ndim = n
        self.num = 1 if n == 1 else n // 3
        self.reso = [int(r) for r in resolution]
        if len(self.reso) != 3:
            raise ValueError("resolution must have 3 entries")
        self.timer = 0.0
        if _handle is None:
            out = C.c_void_p()
            L.call("pvdb_grid_create", L.i32arr(self.reso), n, float(background), C.byref(out))
            _handle = out.value
        self._g = _GridHandle(_handle)

    # ------------------------------------------------------------ handles
    @property
    def handle(self):
        return self._g.h

    @classmethod
    def from_mask(cls, resolution, active, background: float = 0.0, n: int | None = None):
        """Sparse grid: leaves holding at least one active voxel; values = background."""
        n = n if n is not None else (1 if cls is DensityVDB else 12)
        reso = [int(r) for r in resolution]
        out = C.c_void_p()
        if L.is_cuda(active):
            import torch
            a = active.to(torch.uint8).contiguous()
            if a.numel() != reso[0] * reso[1] * reso[2]:
                raise ValueError("active mask size must be prod(resolution)")
            L.call("pvdb_grid_create_from_mask", L.i32arr(reso), n, float(background),
                   L.ptr(a), L.MEM_DEVICE, C.byref(out))
        else:
            a = _as_host_u8(active).reshape(-1)
            if a.size != reso[0] * reso[1] * reso[2]:
                raise ValueError("active mask size must be prod(resolution)")
            L.call("pvdb_grid_create_from_mask", L.i32arr(reso), n, float(background),
                   L.ptr(a), L.MEM_HOST, C.byref(out))
        obj = cls.__new__(cls)
        BaseVDB.__init__(obj, reso, n, _handle=out.value)
        return obj

    # --------------------------------------------------------- reference API
    def getndim(self) -> int:
        return self.ndim

    def getinfo(self):
        print(f"Resolution: ({self.reso[0]},{self.reso[1]},{self.reso[2]})")
        print(f"Num: {self.num}")
        print(f"Dim: {self.ndim}")

    def setReso(self, rx, ry, rz):
        self.reso = [int(rx), int(ry), int(rz)]
        L.call("pvdb_grid_set_reso", self.handle, *self.reso)

    def resetTimer(self):
        self.timer = 0.0

    def getTimer(self) -> float:
        return self.timer

    def info(self):
        """(reso, channels, nleaf, nactive, background)."""
        return _grid_info(self.handle)

    def _nvox(self) -> int:
        return self.reso[0] * self.reso[1] * self.reso[2]

    def forward(self, x, y, z):
        t0 = time.perf_counter()
        if L.is_cuda(x):
            import torch
            xs, ys, zs = _dev_f32(x).reshape(-1), _dev_f32(y).reshape(-1), _dev_f32(z).reshape(-1)
            n = xs.numel()
            if ys.numel() != n or zs.numel() != n:
                raise ValueError("x, y, z must have the same length")
            out = torch.empty(n * self.ndim, device=xs.device, dtype=torch.float32)
            L.call("pvdb_grid_sample", self.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs), n,
                   L.ptr(out), L.MEM_DEVICE, L.stream_of())
        else:
            xs, ys, zs = _as_host_f32(x).reshape(-1), _as_host_f32(y).reshape(-1), _as_host_f32(
                z).reshape(-1)
            n = xs.size
            if ys.size != n or zs.size != n:
                raise ValueError("x, y, z must have the same length")
            out = np.empty(n * self.ndim, np.float32)
            L.call("pvdb_grid_sample", self.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs), n,
                   L.ptr(out), L.MEM_HOST, None)
        self.timer += time.perf_counter() - t0
        return out

    def backward(self, x, y, z, g):
        if L.is_cuda(x):
            xs, ys, zs = _dev_f32(x).reshape(-1), _dev_f32(y).reshape(-1), _dev_f32(z).reshape(-1)
            gg = _dev_f32(g).reshape(-1)
            n = xs.numel()
            if gg.numel() != n * self.ndim:
                raise ValueError("grad must have len(x) * ndim entries")
            L.call("pvdb_grid_sample_backward", self.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs),
                   L.ptr(gg), n, L.MEM_DEVICE, L.stream_of())
        else:
            xs, ys, zs = _as_host_f32(x).reshape(-1), _as_host_f32(y).reshape(-1), _as_host_f32(
                z).reshape(-1)
            gg = _as_host_f32(g).reshape(-1)
            n = xs.size
            if gg.size != n * self.ndim:
                raise ValueError("grad must have len(x) * ndim entries")
            L.call("pvdb_grid_sample_backward", self.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs),
                   L.ptr(gg), n, L.MEM_HOST, None)

    def forward_single(self, i, j, k, with_active: bool = False):
        ii, jj, kk = _as_host_i32(i).reshape(-1), _as_host_i32(j).reshape(-1), _as_host_i32(
            k).reshape(-1)
        n = ii.size
        out = np.empty(n * self.ndim, np.float32)
        act = np.empty(n, np.uint8)
        L.call("pvdb_grid_lookup", self.handle, L.ptr(ii), L.ptr(jj), L.ptr(kk), n, L.ptr(out),
               L.ptr(act), L.MEM_HOST, None)
        return (out, act.astype(bool)) if with_active else out

    def copyFromDense(self, arr, which: int = L.WHICH_DATA):
        if L.is_cuda(arr):
            a = _dev_f32(arr).reshape(-1)
            L.call("pvdb_grid_copy_from_dense", self.handle, which, L.ptr(a), a.numel(),
                   L.MEM_DEVICE, L.stream_of())
        else:
            a = _as_host_f32(arr).reshape(-1)
            L.call("pvdb_grid_copy_from_dense", self.handle, which, L.ptr(a), a.size,
                   L.MEM_HOST, None)

    def get_dense_grid(self, which: int = L.WHICH_DATA, device: bool = False):
        n = self._nvox() * self.ndim
        if device:
            import torch
            out = torch.empty(n, device="cuda", dtype=torch.float32)
            L.call("pvdb_grid_copy_to_dense", self.handle, which, L.ptr(out), n, L.MEM_DEVICE,
                   L.stream_of())
            return out
        out = np.empty(n, np.float32)
        L.call("pvdb_grid_copy_to_dense", self.handle, which, L.ptr(out), n, L.MEM_HOST, None)
        return out

    def total_variation_add_grad(self, wx, wy, wz, dense_mode, mimic_axis_bug: bool = False):
        L.call("pvdb_grid_tv_add_grad", self.handle, float(wx), float(wy), float(wz),
               int(bool(dense_mode)), int(bool(mimic_axis_bug)), L.stream_of())

    def zero_grad(self):
        L.call("pvdb_grid_zero_grad", self.handle, L.stream_of())

    def load_from(self, path: str):
        """Load values (and topology) saved by save_to. When the file has this
        grid's topology the values are copied in place, so optimisers created
        on this grid stay attached (the reference replaces the grid inside the
        same C++ object, plenvdb.h:143-148); a different topology replaces the
        grid and is refused while an optimiser holds it."""
        out = C.c_void_p()
        L.call("pvdb_grid_load", str(path).encode(), C.byref(out))
        new = _GridHandle(out.value)
        reso, ch, nleaf, _, _ = _grid_info(new.h)
        if ch != self.ndim:
            raise ValueError(f"{path} holds {ch} channels, this grid has {self.ndim}")
        if reso == self.reso and _same_topology(self.handle, new.h):
            import torch
            src = _device_arrays(new.h, new)
            dst = _device_arrays(self.handle, self)
            dst["data"].copy_(src["data"])
            torch.cuda.synchronize()
            self.mark_written(L.WHICH_DATA)
            return
        if any(o() is not None for o in getattr(self, "_opts", [])):
            raise ValueError(f"{path} has another topology than this grid and an optimiser is "
                             "attached to it: create the optimiser after loading")
        self._g = new
        self.reso = reso

    def save_to(self, path: str):
        L.call("pvdb_grid_save", self.handle, str(path).encode())

    def device_views(self):
        """Zero-copy torch views: (data [nleaf,512,C], grad [nleaf,512,C], mask [nleaf,8])."""
        d, g, m, t, o = (C.c_void_p() for _ in range(5))
        ld = (C.c_int32 * 3)()
        L.call("pvdb_grid_device_views", self.handle, C.byref(d), C.byref(g), C.byref(m),
               C.byref(t), C.byref(o), ld)
        _, ch, nleaf, _, _ = self.info()
        data = device_view(d.value, (nleaf, 512, ch), "float32", self)
        grad = device_view(g.value, (nleaf, 512, ch), "float32", self)
        mask = device_view(m.value, (nleaf, 8), "uint64", self)
        table = device_view(t.value, tuple(ld), "int32", self)
        origin = device_view(o.value, (nleaf, 3), "int32", self)
        return data, grad, mask, table, origin

    def mark_written(self, which: int = L.WHICH_DATA):
        """Report writes made through views from device_views() after later
        library calls (the data's brick bounds / the touched-leaf tracking)."""
        L.call("pvdb_grid_mark_written", self.handle, int(which))


class DensityVDB(BaseVDB):
    """DensityVDB(resolution, n=1) (plenvdb.h:432-524)."""

    def __init__(self, resolution, n: int = 1, **kw):
        if int(n) != 1:
            raise ValueError("DensityVDB has exactly 1 channel")
        super().__init__(resolution, 1, **kw)

    def setValuesOn_bymask(self, mask, val):
        if L.is_cuda(mask):
            import torch
            m = mask.to(torch.uint8).contiguous().reshape(-1)
            L.call("pvdb_grid_set_values_by_mask", self.handle, L.ptr(m), m.numel(), float(val),
                   L.MEM_DEVICE, L.stream_of())
        else:
            m = _as_host_u8(mask).reshape(-1)
            L.call("pvdb_grid_set_values_by_mask", self.handle, L.ptr(m), m.size, float(val),
                   L.MEM_HOST, None)


class ColorVDB(BaseVDB):
    """ColorVDB(resolution, n=3*num) (plenvdb.h:527-602)."""

    def __init__(self, resolution, n: int, **kw):
        if int(n) <= 0 or int(n) % 3:
            raise ValueError("ColorVDB channels must be a positive multiple of 3")
        super().__init__(resolution, n, **kw)


class _BaseOpt:
    """BaseOptimizer (plenvdb.h:686-744): per-voxel Adam over a VDB's leaves."""

    def __init__(self, vdb: BaseVDB, lr: float, eps: float, beta0: float, beta1: float):
        self.vdb = vdb  # keeps the grid alive (the reference relies on the caller)
        import weakref
        if not hasattr(vdb, "_opts"):
            vdb._opts = []
        vdb._opts.append(weakref.ref(self))
        out = C.c_void_p()
        L.call("pvdb_opt_create", vdb.handle, float(lr), float(eps), float(beta0), float(beta1),
               C.byref(out))
        self.h = out

    def __del__(self):
        try:
            if self.h:
                L.load().pvdb_opt_destroy(self.h)
                self.h = C.c_void_p(None)
        except Exception:
            pass

    def step(self, mode: int = 0, zero_grad_after: bool = False):
        L.call("pvdb_opt_step", self.h, int(mode), int(bool(zero_grad_after)), L.stream_of())

    def zero_grad(self):
        L.call("pvdb_opt_zero_grad", self.h, L.stream_of())

    def set_grad(self, arr):
        if L.is_cuda(arr):
            a = _dev_f32(arr).reshape(-1)
            L.call("pvdb_opt_set_grad", self.h, L.ptr(a), a.numel(), L.MEM_DEVICE, L.stream_of())
        else:
            a = _as_host_f32(arr).reshape(-1)
            L.call("pvdb_opt_set_grad", self.h, L.ptr(a), a.size, L.MEM_HOST, None)

    def set_pervoxel_lr(self, count):
        if L.is_cuda(count):
            a = _dev_f32(count).reshape(-1)
            L.call("pvdb_opt_set_pervoxel_lr", self.h, L.ptr(a), a.numel(), L.MEM_DEVICE,
                   L.stream_of())
        else:
            a = _as_host_f32(count).reshape(-1)
            L.call("pvdb_opt_set_pervoxel_lr", self.h, L.ptr(a), a.size, L.MEM_HOST, None)

    def update_lr(self, factor):
        L.call("pvdb_opt_update_lr", self.h, float(factor))

    def _scalars(self):
        st = C.c_int32()
        lr, eps, b0, b1 = C.c_float(), C.c_float(), C.c_float(), C.c_float()
        L.call("pvdb_opt_get_scalars", self.h, C.byref(st), C.byref(lr), C.byref(eps),
               C.byref(b0), C.byref(b1))
        return st.value, lr.value, eps.value, b0.value, b1.value

    def _set(self, **kw):
        st, lr, eps, b0, b1 = self._scalars()
        st = kw.get("step", st)
        lr = kw.get("lr", lr)
        eps = kw.get("eps", eps)
        b0 = kw.get("b0", b0)
        b1 = kw.get("b1", b1)
        L.call("pvdb_opt_set_scalars", self.h, int(st), float(lr), float(eps), float(b0), float(b1))

    def getStep(self):
        return self._scalars()[0]

    def getLr(self):
        return self._scalars()[1]

    def getEps(self):
        return self._scalars()[2]

    def getBeta0(self):
        return self._scalars()[3]

    def getBeta1(self):
        return self._scalars()[4]

    def setStep(self, x):
        self._set(step=x)

    def setLr(self, x):
        self._set(lr=x)

    def setEps(self, x):
        self._set(eps=x)

    def setBeta0(self, x):
        self._set(b0=x)

    def setBeta1(self, x):
        self._set(b1=x)

    def getinfo(self):
        r = self.vdb.reso
        st, lr, eps, b0, b1 = self._scalars()
        print(f"Resolution: ({r[0]},{r[1]},{r[2]})")
        print(f"Num: {self.vdb.num}")
        print(f"Dim: {self.vdb.ndim}")
        print(f"Step: {st}")
        print(f"lr: {lr}")
        print(f"eps: {eps}")
        print(f"beta: {b0},{b1}")

    def _moments(self):
        a, b = C.c_void_p(), C.c_void_p()
        L.call("pvdb_opt_moments", self.h, C.byref(a), C.byref(b))
        return a, b

    def save_to(self, prefix: str):
        a, b = self._moments()
        L.call("pvdb_grid_save", a, (str(prefix) + "exp_avg.vdb").encode())
        L.call("pvdb_grid_save", b, (str(prefix) + "exp_avg_sq.vdb").encode())

    def load_from(self, prefix: str):
        import torch
        for dst, name in zip(self._moments(), ("exp_avg.vdb", "exp_avg_sq.vdb")):
            out = C.c_void_p()
            L.call("pvdb_grid_load", (str(prefix) + name).encode(), C.byref(out))
            src = _GridHandle(out.value)
            _, ch_s, nl_s, _, _ = _grid_info(src.h)
            _, ch_d, nl_d, _, _ = _grid_info(dst)
            if (ch_s, nl_s) != (ch_d, nl_d):
                raise ValueError(f"{prefix}{name}: topology differs from the optimiser's grid")
            ptrs = []
            for h in (src.h, dst):
                d = C.c_void_p()
                L.call("pvdb_grid_device_views", h, C.byref(d), None, None, None, None, None)
                ptrs.append(d.value)
            n = nl_s * 512 * ch_s
            s_t = device_view(ptrs[0], (n,), "float32", src)
            d_t = device_view(ptrs[1], (n,), "float32", self)
            d_t.copy_(s_t)
            torch.cuda.synchronize()


class DensityOpt(_BaseOpt):
    """DensityOpt(vdb, lr, eps, beta0, beta1) (plenvdb.h:747-768)."""


class ColorOpt(_BaseOpt):
    """ColorOpt(vdb, lr, eps, beta0, beta1) (plenvdb.h:770-790)."""


def _renderer_cls():
    from .renderer import MGRenderer
    return MGRenderer


def __getattr__(name):
    if name == "MGRenderer":
        return _renderer_cls()
    raise AttributeError(name)
