"""The DVGO schedule around the training step, on the leaf store and libpvdb's
CUDA kernels:

* ``MaskGrid`` — the mask cache (lib/grid.py:207-246), with its three builds:
  from a checkpoint's density (``MaskGrid(path=...)`` / ``mask_from_density``,
  grid.py:210-221), ``update_occupancy_cache`` (lib/dvgo.py:200-210) and the
  rebuild after progressive scaling (``rescaled_mask_cache``, dvgo.py:186-197);
* ``scale_volume_grid`` (VDBGrid.scale_volume_grid, lib/grid.py:91-102);
* ``maskout_near_cam_vox`` (lib/dvgo.py:163-175);
* ``voxel_count_views`` (lib/dvgo.py:212-243), the per-voxel lr counts;
* the merged-row compression of a trained model for MGRenderer
  (vdb_compression.py:19-59) and its on-disk form (``save_merged`` /
  ``load_merged``; mergeddata.npz keeps the reference's keys and FP16 rows,
  mergedidxs.npz replaces the OpenVDB index grid mergedidxs.vdb with the
  packed occupancy bits the row ids follow from).

Grids are ``DensityVDB`` / ``ColorVDB``; masks are CUDA uint8/bool tensors.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import _lib as L
from . import render_utils as RU
from .plenvdb import ColorVDB, DensityVDB


def _vec3(v) -> list[float]:
    if torch.is_tensor(v):
        v = v.detach().float().cpu().reshape(-1).tolist()
    return [float(x) for x in np.asarray(v, np.float32).reshape(-1)]


def _mask_u8(mask) -> torch.Tensor:
    if not torch.is_tensor(mask):
        mask = torch.from_numpy(np.ascontiguousarray(np.asarray(mask)))
    return mask.to(device="cuda", dtype=torch.uint8).contiguous()


# ------------------------------------------------------------ mask cache
class MaskGrid:
    """MaskGrid (lib/grid.py:207-246). ``mask`` is a CUDA uint8 tensor of the
    mask-cache shape; ``__call__(xyz)`` is the nearest lookup of
    maskcache_lookup with the reference's scale/shift buffers.

    ``path`` is a checkpoint written by ``FineStageTrainer.save_checkpoint``
    (``<prefix>last.npz``): as in the reference, its density grid sits at
    ``path[:-9] + 'density.pvdb'`` and the mask is
    ``1 - exp(-softplus(maxpool3(density) + act_shift) * voxel_size_ratio) >= mask_cache_thres``."""

    def __init__(self, path=None, mask_cache_thres=None, mask=None, xyz_min=None, xyz_max=None):
        if path is not None:
            st = np.load(path)
            density = DensityVDB([2, 2, 2], 1)
            density.load_from(path[:-9] + "density.pvdb")
            xyz_min = st["xyz_min"].astype(np.float32)
            xyz_max = st["xyz_max"].astype(np.float32)
            mask = mask_from_density(density, float(st["act_shift"]),
                                     float(st["voxel_size_ratio"]), float(mask_cache_thres),
                                     xyz_min, xyz_max)
        self.mask = _mask_u8(mask)
        self.xyz_min = _vec3(xyz_min)
        self.xyz_max = _vec3(xyz_max)
        shape = np.array(self.mask.shape, np.float32)
        ext = np.array(self.xyz_max, np.float32) - np.array(self.xyz_min, np.float32)
        self.xyz2ijk_scale = ((shape - np.float32(1)) / ext).astype(np.float32)
        self.xyz2ijk_shift = (-np.array(self.xyz_min, np.float32) * self.xyz2ijk_scale).astype(
            np.float32)

    @property
    def shape(self):
        return tuple(self.mask.shape)

    @torch.no_grad()
    def __call__(self, xyz):
        shape = xyz.shape[:-1]
        out = RU.maskcache_lookup(self.mask, xyz.reshape(-1, 3), self.xyz2ijk_scale,
                                  self.xyz2ijk_shift)
        return out.reshape(shape)

    forward = __call__


def _occupancy(density, mode, mask, xyz_min, xyz_max, act_shift, interval, thres,
               old_mask=None):
    shape = list(mask.shape)
    old_shape = L.i32arr(list(old_mask.shape)) if old_mask is not None else None
    L.call("pvdb_occupancy", density.handle, int(mode), L.ptr(mask), L.i32arr(shape),
           L.f32arr(_vec3(xyz_min)), L.f32arr(_vec3(xyz_max)), float(act_shift),
           float(interval), float(thres), L.ptr(old_mask), old_shape, L.stream_of())


def mask_from_density(density: DensityVDB, act_shift, voxel_size_ratio, mask_cache_thres,
                      xyz_min, xyz_max) -> torch.Tensor:
    """The mask of MaskGrid(path=...) (lib/grid.py:214-221) over the grid's voxels."""
    mask = torch.empty(density.reso, device="cuda", dtype=torch.uint8)
    _occupancy(density, 2, mask, xyz_min, xyz_max, act_shift, voxel_size_ratio,
               mask_cache_thres)
    return mask


@torch.no_grad()
def update_occupancy_cache(mask_cache: MaskGrid, density: DensityVDB, act_shift, interval,
                           fast_color_thres):
    """DirectVoxGO.update_occupancy_cache (lib/dvgo.py:200-210), in place."""
    _occupancy(density, 0, mask_cache.mask, mask_cache.xyz_min, mask_cache.xyz_max, act_shift,
               interval, fast_color_thres)
    return mask_cache


@torch.no_grad()
def rescaled_mask_cache(mask_cache: MaskGrid | None, density: DensityVDB, xyz_min, xyz_max,
                        act_shift, interval, fast_color_thres) -> MaskGrid:
    """The mask cache that scale_volume_grid builds for the new resolution
    (lib/dvgo.py:186-197): the old cache looked up at the new grid points, and
    maxpool3(alpha(density)) > fast_color_thres."""
    mask = torch.empty(density.reso, device="cuda", dtype=torch.uint8)
    _occupancy(density, 1, mask, xyz_min, xyz_max, act_shift, interval, fast_color_thres,
               old_mask=None if mask_cache is None else mask_cache.mask)
    return MaskGrid(mask=mask, xyz_min=xyz_min, xyz_max=xyz_max)


# ------------------------------------------------------------ rescaling
@torch.no_grad()
def scale_volume_grid(vdb, new_world_size):
    """VDBGrid.scale_volume_grid (lib/grid.py:91-102): a new dense grid of
    ``new_world_size`` holding F.interpolate(trilinear, align_corners=True) of
    ``vdb``'s values; returns it (the reference swaps it into the module)."""
    ws = [int(v) for v in (new_world_size.tolist() if torch.is_tensor(new_world_size)
                           else new_world_size)]
    cls = DensityVDB if vdb.ndim == 1 else ColorVDB
    new = cls(ws, vdb.ndim)
    L.call("pvdb_grid_resample", vdb.handle, new.handle, L.stream_of())
    return new


@torch.no_grad()
def maskout_near_cam_vox(density: DensityVDB, cam_o, near_clip, xyz_min, xyz_max,
                         value: float = -100.0):
    """DirectVoxGO.maskout_near_cam_vox (lib/dvgo.py:163-175)."""
    cams = torch.as_tensor(cam_o).to(device="cuda", dtype=torch.float32).reshape(-1, 3)
    cams = cams.contiguous()
    L.call("pvdb_grid_maskout_near_cams", density.handle, L.ptr(cams), cams.shape[0],
           L.f32arr(_vec3(xyz_min)), L.f32arr(_vec3(xyz_max)), float(near_clip), float(value),
           L.stream_of())


@torch.no_grad()
def voxel_count_views(rays_o_tr, rays_d_tr, imsz, near, far, stepsize, world_size, voxel_size,
                      xyz_min, xyz_max, downrate=1, irregular_shape=False):
    """DirectVoxGO.voxel_count_views (lib/dvgo.py:212-243): for each view, the
    voxels whose summed trilinear weight over the view's ray samples exceeds 1
    count the view. Returns count [1,1,X,Y,Z] (float32, CUDA)."""
    ws = [int(v) for v in (world_size.tolist() if torch.is_tensor(world_size) else world_size)]
    n_samples = int(np.linalg.norm(np.array(ws) + 1) / stepsize) + 1
    # stepsize * voxel_size as the reference's float32 tensor product
    stepdist = float(np.float32(stepsize) * np.float32(voxel_size))
    count = torch.zeros([1, 1] + ws, device="cuda", dtype=torch.float32)
    acc = torch.zeros(ws, device="cuda", dtype=torch.int64)
    for rays_o_, rays_d_ in zip(rays_o_tr.split(imsz), rays_d_tr.split(imsz)):
        if not irregular_shape:
            rays_o_ = rays_o_[::downrate, ::downrate]
            rays_d_ = rays_d_[::downrate, ::downrate]
        ro = rays_o_.to(device="cuda", dtype=torch.float32).reshape(-1, 3).contiguous()
        rd = rays_d_.to(device="cuda", dtype=torch.float32).reshape(-1, 3).contiguous()
        L.call("pvdb_count_views", L.ptr(ro), L.ptr(rd), ro.shape[0], L.i32arr(ws),
               L.f32arr(_vec3(xyz_min)), L.f32arr(_vec3(xyz_max)), float(near), stepdist,
               n_samples, L.ptr(acc), L.ptr(count), L.stream_of())
    return count


# ------------------------------------------------------ merged compression
_ROW_DTYPES = {"float32": (0, torch.float32), "float16": (1, torch.float16)}


@torch.no_grad()
def merge_compress(density: DensityVDB | None, color: ColorVDB | None, mask,
                   row_dtype: str = "float16"):
    """vdb_compression.py:19-59 on the device: row ids 1..N for the masked
    voxels in C order (0 = empty), and the density / colour rows (row 0 zero).
    Returns dict(index [rx,ry,rz] int32, den [N+1], col [N+1, C], N=N+1)."""
    ref = density if density is not None else color
    m = _mask_u8(mask).reshape(-1)
    if m.numel() != ref.reso[0] * ref.reso[1] * ref.reso[2]:
        raise ValueError("mask size must be the grids' voxel count")
    code, tdt = _ROW_DTYPES[row_dtype]
    n = C.c_int64()
    L.call("pvdb_merge_count", L.ptr(m), m.numel(), C.byref(n), L.stream_of())
    rows = n.value + 1
    index = torch.empty(ref.reso, device="cuda", dtype=torch.int32)
    den = torch.empty(rows, device="cuda", dtype=tdt) if density is not None else None
    col = (torch.empty(rows, color.ndim, device="cuda", dtype=tdt) if color is not None
           else None)
    L.call("pvdb_merge_build", None if density is None else density.handle,
           None if color is None else color.handle, L.ptr(m), L.ptr(index), L.ptr(den),
           L.ptr(col), rows, code, L.stream_of())
    return {"index": index, "den": den, "col": col, "N": rows}


def save_merged(ckptdir: str, merged) -> None:
    """mergeddata.npz (keys den, col; FP16 rows as vdb_compression.py:55-58)
    and mergedidxs.npz (resolution + packed occupancy bits in C order)."""
    den = merged["den"].cpu().numpy()
    col = merged["col"].cpu().numpy()
    np.savez_compressed(os.path.join(ckptdir, "mergeddata"), den=den, col=col)
    occ = (merged["index"] > 0).cpu().numpy().reshape(-1)
    np.savez_compressed(os.path.join(ckptdir, "mergedidxs"),
                        reso=np.array(merged["index"].shape, np.int32), bits=np.packbits(occ))


def load_merged_index(path: str) -> np.ndarray:
    """The dense int32 row-id grid [rx,ry,rz] of a mergedidxs.npz."""
    z = np.load(path)
    reso = [int(r) for r in z["reso"]]
    n = reso[0] * reso[1] * reso[2]
    occ = np.unpackbits(z["bits"], count=n).astype(bool)
    index = np.zeros(n, np.int32)
    index[occ] = np.arange(1, int(occ.sum()) + 1, dtype=np.int32)
    return index.reshape(reso)


def load_merged(ckptdir: str):
    """(den [N] f32, col [N*C] f32, index [rx,ry,rz] int32, N) as run.py's
    create_renderer reads them (run.py:83-91)."""
    vdbdata = np.load(os.path.join(ckptdir, "mergeddata.npz"))
    den = vdbdata["den"].astype(np.float32)
    col = vdbdata["col"].astype(np.float32)
    index = load_merged_index(os.path.join(ckptdir, "mergedidxs.npz"))
    return den.reshape(-1), col.reshape(-1), index, den.shape[0]
