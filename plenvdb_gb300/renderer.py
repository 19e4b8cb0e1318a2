"""MGRenderer — merged-VDB inference renderer with the reference's method
names (plenvdb.h:933-1068, bound at plenvdb.cpp:135-170)."""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _lib as L


class MGRenderer:
    def __init__(self, dcol: int, dpe: int, dhid: int, dout: int):
        out = C.c_void_p()
        L.call("pvdb_renderer_create", int(dcol), int(dpe), int(dhid), int(dout), C.byref(out))
        self.h = out
        self.dcol, self.dpe, self.dhid, self.dout = dcol, dpe, dhid, dout
        self.timer = 0.0
        self.t_stop = 1e-3
        self.precision = 0
        self._hw = None

    def __del__(self):
        try:
            if self.h:
                L.load().pvdb_renderer_destroy(self.h)
                self.h = C.c_void_p(None)
        except Exception:
            pass

    def load_data(self, den, col, index, N, reso=None, storage: int = 0):
        """load_data(den [N], col [N*dcol], index, N): `index` is a dense int array of
        row ids [rx,ry,rz] (0 = empty) or the path of a mergedidxs.npz written by
        lifecycle.save_merged. The reference reads an OpenVDB index grid from a
        .vdb path here; that format is not supported."""
        if isinstance(index, (str, bytes, os.PathLike)):
            path = os.fsdecode(index)
            if not path.endswith(".npz"):
                raise ValueError("OpenVDB .vdb index grids are not supported: pass the dense "
                                 "row-id array or a mergedidxs.npz from lifecycle.save_merged")
            from .lifecycle import load_merged_index
            index = load_merged_index(path)
        idx = np.ascontiguousarray(np.asarray(index), np.int32)
        reso = list(idx.shape) if reso is None else [int(r) for r in reso]
        den = np.ascontiguousarray(np.asarray(den, np.float32).reshape(-1))
        col = np.ascontiguousarray(np.asarray(col, np.float32).reshape(-1))
        if den.size != int(N) or col.size != int(N) * self.dcol:
            raise ValueError("den must have N entries and col N*dcol entries")
        L.call("pvdb_renderer_load_data", self.h, L.i32arr(reso), L.ptr(idx.reshape(-1)),
               L.ptr(den), L.ptr(col), int(N), int(storage), L.MEM_HOST)

    def load_params(self, w0, b0, w1, b1, w2, b2):
        arrs = [np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1)) for a in
                (w0, b0, w1, b1, w2, b2)]
        L.call("pvdb_renderer_load_params", self.h, *[L.ptr(a) for a in arrs])

    def setScene(self, reso, K, xyz_min, xyz_max):
        L.call("pvdb_renderer_set_scene", self.h, L.i32arr(reso),
               L.f32arr(np.asarray(K, np.float32).reshape(-1)), L.f32arr(xyz_min), L.f32arr(xyz_max))

    def setKwargs(self, near, far, stepdist, act_shift, interval, fast_color_thres, bg, inverse_y,
                  h, w, t_stop: float | None = None):
        if t_stop is not None:
            self.t_stop = float(t_stop)
        L.call("pvdb_renderer_set_kwargs", self.h, float(near), float(far), float(stepdist),
               float(act_shift), float(interval), float(fast_color_thres), float(bg),
               int(bool(inverse_y)), int(h), int(w), float(self.t_stop))
        self._hw = (int(h), int(w))

    def input_a_c2w(self, c2w):
        if L.is_cuda(c2w):
            t = c2w.float().contiguous()
            L.call("pvdb_renderer_input_c2w", self.h, L.ptr(t), L.MEM_DEVICE, L.stream_of())
        else:
            a = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(-1))
            L.call("pvdb_renderer_input_c2w", self.h, L.ptr(a), L.MEM_HOST, None)

    def render_an_image(self):
        t0 = time.perf_counter()
        L.call("pvdb_renderer_render", self.h, int(self.precision), L.stream_of())
        self.timer += time.perf_counter() - t0

    def output_an_image(self, device: bool = False):
        H, W = self._hw
        if device:
            import torch
            out = torch.empty(H * W * 3, device="cuda", dtype=torch.float32)
            L.call("pvdb_renderer_output", self.h, L.ptr(out), L.MEM_DEVICE, L.stream_of())
            return out
        out = np.empty(H * W * 3, np.float32)
        L.call("pvdb_renderer_output", self.h, L.ptr(out), L.MEM_HOST, L.stream_of())
        return out

    def resetTimer(self):
        self.timer = 0.0

    def getTimer(self) -> float:
        return self.timer
