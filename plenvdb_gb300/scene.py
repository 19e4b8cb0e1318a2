"""Seeded synthetic scenes, cameras and rays standing in for the NeRF-synthetic
data the reference trains on (no dataset is available here).

Scene: a bbox [-1.5, 1.5]^3 voxelised at `reso`^3 with the reference's
align_corners index mapping (grid.py:77-78); the union of `n_ellipsoids`
axis-aligned ellipsoids (centres U[-1,1]^3, radii U[0.15,0.5]) and, optionally,
a thin spherical shell |‖x‖ - 1.3| < 0.02. Active voxels are the voxels whose
centre lies inside; leaves holding any active voxel are allocated; inactive
and out-of-leaf values read the background -10. Raw density N(2,1) and k0
features N(0,0.1) on the active voxels.

Cameras: uniform on the sphere of radius 4.03 looking at the origin,
800x800 with focal 1111.1 (get_rays convention of dvgo.py:471-501,
inverse_y=False).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class SceneConfig:
    reso: int = 160
    n_ellipsoids: int = 8
    shell: bool = False
    seed: int = 0
    k0_dim: int = 12
    bbox: float = 1.5
    background: float = -10.0
    density_mean: float = 2.0
    density_std: float = 1.0
    k0_std: float = 0.1

    @property
    def xyz_min(self):
        return [-self.bbox] * 3

    @property
    def xyz_max(self):
        return [self.bbox] * 3


def voxel_world(cfg: SceneConfig, idx: np.ndarray) -> np.ndarray:
    """World position of voxel indices (inverse of wld2idx)."""
    return -cfg.bbox + idx.astype(np.float64) / (cfg.reso - 1) * (2 * cfg.bbox)


def scene_mask(cfg: SceneConfig) -> np.ndarray:
    """Active mask [R,R,R] (uint8)."""
    rng = np.random.default_rng(cfg.seed)
    R = cfg.reso
    centres = rng.uniform(-1, 1, (cfg.n_ellipsoids, 3))
    radii = rng.uniform(0.15, 0.5, (cfg.n_ellipsoids, 3))
    active = np.zeros((R, R, R), np.uint8)
    coords = voxel_world(cfg, np.arange(R))
    for c, r in zip(centres, radii):
        lo = np.searchsorted(coords, c - r, side="left")
        hi = np.searchsorted(coords, c + r, side="right")
        xs, ys, zs = (coords[lo[a]:hi[a]] for a in range(3))
        if not (len(xs) and len(ys) and len(zs)):
            continue
        d = (((xs[:, None, None] - c[0]) / r[0]) ** 2 + ((ys[None, :, None] - c[1]) / r[1]) ** 2 +
             ((zs[None, None, :] - c[2]) / r[2]) ** 2)
        active[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] |= (d <= 1.0).astype(np.uint8)
    if cfg.shell:
        for i in range(R):
            x = coords[i]
            d = np.sqrt(x * x + coords[:, None] ** 2 + coords[None, :] ** 2)
            active[i] |= (np.abs(d - 1.3) < 0.02).astype(np.uint8)
    return active


def scene_dense(cfg: SceneConfig, value_seed: int | None = None):
    """(active [R^3] u8, density [R^3] f32, k0 [R^3, C] f32) as dense arrays."""
    active = scene_mask(cfg)
    rng = np.random.default_rng(cfg.seed + 1000 if value_seed is None else value_seed)
    R = cfg.reso
    dens = rng.normal(cfg.density_mean, cfg.density_std, (R, R, R)).astype(np.float32)
    dens = np.where(active > 0, dens, np.float32(cfg.background)).astype(np.float32)
    k0 = rng.normal(0.0, cfg.k0_std, (R, R, R, cfg.k0_dim)).astype(np.float32)
    k0 *= (active > 0)[..., None]
    return active, dens, k0


def build_grids(cfg: SceneConfig, value_seed: int | None = None, device_fill: bool | None = None):
    """DensityVDB + ColorVDB with the scene's sparse topology and values.

    Small scenes go through dense arrays (copyFromDense); large ones are filled
    on the device through the leaf-store views with a seeded torch generator."""
    import torch

    from .plenvdb import ColorVDB, DensityVDB
    if device_fill is None:
        device_fill = cfg.reso > 192
    reso = [cfg.reso] * 3
    if not device_fill:
        active, dens, k0 = scene_dense(cfg, value_seed)
        dg = DensityVDB.from_mask(reso, active, background=cfg.background)
        kg = ColorVDB.from_mask(reso, active, background=0.0, n=cfg.k0_dim)
        dg.copyFromDense(dens.reshape(-1))
        kg.copyFromDense(k0.reshape(-1))
        return dg, kg
    active = scene_mask(cfg)
    dg = DensityVDB.from_mask(reso, active, background=cfg.background)
    kg = ColorVDB.from_mask(reso, active, background=0.0, n=cfg.k0_dim)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(cfg.seed + 1000 if value_seed is None else value_seed)
    d_data, _, d_mask, _, _ = dg.device_views()
    k_data, _, _, _, _ = kg.device_views()
    bits = torch.arange(64, device="cuda", dtype=torch.int64)
    act = ((d_mask.view(torch.int64).unsqueeze(-1) >> bits) & 1).reshape(-1, 512).bool()
    vals = torch.randn(d_data.shape[0], 512, generator=gen, device="cuda") * cfg.density_std + \
        cfg.density_mean
    d_data[..., 0].copy_(torch.where(act, vals, torch.full_like(vals, cfg.background)))
    feats = torch.randn(k_data.shape, generator=gen, device="cuda") * cfg.k0_std
    k_data.copy_(feats * act.unsqueeze(-1))
    torch.cuda.synchronize()
    return dg, kg


# --------------------------------------------------------------- cameras
@dataclass
class CameraConfig:
    H: int = 800
    W: int = 800
    focal: float = 1111.1
    radius: float = 4.03
    near: float = 2.0
    far: float = 6.0
    inverse_y: bool = False

    @property
    def K(self):
        return np.array([[self.focal, 0, self.W / 2], [0, self.focal, self.H / 2], [0, 0, 1]],
                        np.float32)


def look_at_c2w(pos: np.ndarray) -> np.ndarray:
    """Camera-to-world 4x4 for a camera at pos looking at the origin (+z up)."""
    back = pos / np.linalg.norm(pos)
    up0 = np.array([0.0, 0.0, 1.0]) if abs(back[2]) < 0.999 else np.array([0.0, 1.0, 0.0])
    right = np.cross(up0, back)
    right /= np.linalg.norm(right)
    up = np.cross(back, right)
    c2w = np.eye(4)
    c2w[:3, 0], c2w[:3, 1], c2w[:3, 2], c2w[:3, 3] = right, up, back, pos
    return c2w.astype(np.float32)


def sphere_poses(n: int, radius: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return np.stack([look_at_c2w(radius * p) for p in v])


def spiral_poses(n: int, radius: float, elevation_deg: float, seed: int = 0) -> np.ndarray:
    """Render path: azimuth sweep at a fixed elevation (cf. load_blender.py:74)."""
    rng = np.random.default_rng(seed)
    phase = rng.uniform(0, 2 * np.pi)
    el = np.deg2rad(elevation_deg)
    out = []
    for t in np.linspace(0, 2 * np.pi, n, endpoint=False):
        az = t + phase
        pos = radius * np.array([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), -np.sin(el)])
        out.append(look_at_c2w(pos))
    return np.stack(out)


def rays_of_pixels(cam: CameraConfig, c2w: np.ndarray, px: np.ndarray, py: np.ndarray):
    """get_rays (dvgo.py:471-501) for selected pixels: (rays_o, rays_d, viewdirs) float32."""
    K = cam.K
    i = px.astype(np.float32) + np.float32(0.5)
    j = py.astype(np.float32) + np.float32(0.5)
    if cam.inverse_y:
        dirs = np.stack([(i - K[0][2]) / K[0][0], (j - K[1][2]) / K[1][1], np.ones_like(i)], -1)
    else:
        dirs = np.stack([(i - K[0][2]) / K[0][0], -(j - K[1][2]) / K[1][1], -np.ones_like(i)], -1)
    dirs = dirs.astype(np.float32)
    rot = c2w[:3, :3].astype(np.float32)
    rays_d = (dirs[..., None, :] * rot).sum(-1).astype(np.float32)
    rays_o = np.broadcast_to(c2w[:3, 3].astype(np.float32), rays_d.shape).copy()
    viewdirs = (rays_d / np.linalg.norm(rays_d, axis=-1, keepdims=True)).astype(np.float32)
    return rays_o, rays_d, viewdirs


def random_rays(cam: CameraConfig, n_rays: int, n_views: int, seed: int):
    """n_rays rays drawn uniformly over (view, pixel) of n_views seeded cameras."""
    rng = np.random.default_rng(seed)
    poses = sphere_poses(n_views, cam.radius, seed + 7)
    view = rng.integers(0, n_views, n_rays)
    px = rng.integers(0, cam.W, n_rays)
    py = rng.integers(0, cam.H, n_rays)
    o = np.empty((n_rays, 3), np.float32)
    d = np.empty((n_rays, 3), np.float32)
    v = np.empty((n_rays, 3), np.float32)
    for k in range(n_views):
        sel = view == k
        if sel.any():
            o[sel], d[sel], v[sel] = rays_of_pixels(cam, poses[k], px[sel], py[sel])
    return o, d, v


def rgbnet_init(c0: int = 12, pe: int = 4, width: int = 128, seed: int = 0):
    """rgbnet weights with torch's nn.Linear default init, final bias 0 (dvgo.py:99-107)."""
    import torch
    g = torch.Generator().manual_seed(seed)
    din = c0 + 3 + 6 * pe
    out = []
    for fan_in, fan_out in ((din, width), (width, width), (width, 3)):
        bound = 1.0 / np.sqrt(fan_in)
        w = (torch.rand(fan_out, fan_in, generator=g) * 2 - 1) * bound
        b = (torch.rand(fan_out, generator=g) * 2 - 1) * bound
        out += [w, b]
    out[-1].zero_()
    return out  # [w0, b0, w1, b1, w2, b2] in nn.Linear [out, in] layout
