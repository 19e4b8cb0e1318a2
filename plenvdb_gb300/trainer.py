"""Fine-stage trainer over the native fused step (pvdb_train_step).

One call of ``FineStageTrainer.step`` is one iteration of the reference's
scene_rep_reconstruction loop body (run.py:516-598): forward, losses (MSE,
entropy of alphainv_last, per-point rgb), backward, TV, voxel Adam on both
grids with skip-zero-grad (configs/default.py:76), Adam on the rgbnet, lr
decay by 0.1^(1/(lrate_decay*1000)). Rays, targets and every intermediate stay
on the device; the step never synchronises with the host.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from .march import MarchWorkspace, march_params
from .plenvdb import ColorOpt, DensityOpt


@dataclass
class FineStageConfig:
    xyz_min: tuple = (-1.5, -1.5, -1.5)
    xyz_max: tuple = (1.5, 1.5, 1.5)
    reso: int = 160
    stepsize: float = 0.5           # voxels per step (configs/default.py:103)
    near: float = 2.0
    bg: float = 0.0
    act_shift: float = -4.6
    interval: float = 0.5           # stepsize * voxel_size_ratio
    fast_color_thres: float = 1e-4
    t_stop: float = 1e-3
    lr_density: float = 0.1
    lr_k0: float = 0.075
    lr_rgbnet: float = 1e-3
    lrate_decay: int = 20
    betas: tuple = (0.9, 0.99)
    eps: float = 1e-8
    weight_main: float = 1.0
    weight_entropy_last: float = 1e-3
    weight_rgbper: float = 1e-2
    tv_weight: float = 1e-4
    tv_dense_mode: bool = False
    precision: int = 0              # 0 FP32 SIMT rgbnet, 1 BF16 tensor cores
    use_graph: bool = True          # replay the fused step as a captured CUDA graph
    leaf_staging: bool = False      # density leaves staged in shared memory by bulk copies
    tv_in_place: bool = False       # sparse TV added to the gradient before Adam, not deferred

    @property
    def voxel_size(self) -> float:
        ext = np.array(self.xyz_max, np.float64) - np.array(self.xyz_min, np.float64)
        return float((ext.prod() / self.reso ** 3) ** (1 / 3))

    @property
    def stepdist(self) -> float:
        return self.stepsize * self.voxel_size


class FineStageTrainer:
    def __init__(self, density, k0, rgbnet_params, cfg: FineStageConfig, max_rays: int):
        self.cfg = cfg
        self.density, self.k0 = density, k0
        b0, b1 = cfg.betas
        self.dopt = DensityOpt(density, cfg.lr_density, cfg.eps, b0, b1)
        self.kopt = ColorOpt(k0, cfg.lr_k0, cfg.eps, b0, b1)
        self.ws = MarchWorkspace(max_rays, cfg.xyz_min, cfg.xyz_max, cfg.stepdist,
                                 leaf_staging=cfg.leaf_staging)
        w0, b0_, w1, b1_, w2, b2 = rgbnet_params
        self.c0 = k0.ndim
        self.pe = (w0.shape[1] - self.c0 - 3) // 6
        flat = torch.cat([t.reshape(-1).float() for t in (w0, b0_, w1, b1_, w2, b2)])
        self.params = flat.cuda().contiguous()
        self.grads = torch.zeros_like(self.params)
        self.exp_avg = torch.zeros_like(self.params)
        self.exp_avg_sq = torch.zeros_like(self.params)
        self._step = C.c_int32(0)
        self._lr = C.c_float(cfg.lr_rgbnet)
        self.state = L.RgbnetState()
        self.state.params, self.state.grads = L.ptr(self.params), L.ptr(self.grads)
        self.state.exp_avg, self.state.exp_avg_sq = L.ptr(self.exp_avg), L.ptr(self.exp_avg_sq)
        self.state.step = C.pointer(self._step)
        self.state.lr = C.pointer(self._lr)
        self.state.c0, self.state.pe, self.state.width = self.c0, self.pe, w1.shape[0]
        self.tc = L.TrainConfig()
        self.tc.march = march_params(cfg.xyz_min, cfg.xyz_max, cfg.near, cfg.stepdist,
                                     cfg.act_shift, cfg.interval, cfg.fast_color_thres, cfg.bg,
                                     cfg.t_stop)
        self.tc.weight_main = cfg.weight_main
        self.tc.weight_entropy_last = cfg.weight_entropy_last
        self.tc.weight_rgbper = cfg.weight_rgbper
        self.tc.tv_weight_density = cfg.tv_weight
        self.tc.tv_weight_k0 = cfg.tv_weight
        self.tc.tv_dense_mode = int(cfg.tv_dense_mode)
        self.tc.lr_decay_factor = 0.1 ** (1.0 / (cfg.lrate_decay * 1000))
        self.tc.rgbnet_lr = cfg.lr_rgbnet
        self.tc.rgbnet_beta1, self.tc.rgbnet_beta2 = cfg.betas
        self.tc.rgbnet_eps = cfg.eps
        self.tc.precision = cfg.precision
        # bytes per k0 feature the BF16 step gathers (its 12-channel BF16 shadow)
        self.k0_feature_bytes = 2 if (cfg.precision == 1 and self.c0 == 12) else 4
        self.tc.use_graph = int(cfg.use_graph)
        self.tc.tv_in_place = int(cfg.tv_in_place)
        self.loss = torch.zeros(1, device="cuda")
        # gradients start clean
        density.zero_grad()
        k0.zero_grad()

    def rgbnet_tensors(self):
        """Views [w0, b0, w1, b1, w2, b2] of the flat rgbnet parameters."""
        W, din = 128, self.c0 + 3 + 6 * self.pe
        sizes = [(W, din), (W,), (W, W), (W,), (3, W), (3,)]
        out, o = [], 0
        for s in sizes:
            n = int(np.prod(s))
            out.append(self.params[o:o + n].view(*s))
            o += n
        return out

    def step(self, rays_o, rays_d, viewdirs, target):
        n = rays_o.shape[0]
        L.call("pvdb_train_step", self.ws.h, self.dopt.h, self.kopt.h, C.byref(self.state),
               L.ptr(rays_o), L.ptr(rays_d), L.ptr(viewdirs), L.ptr(target), n,
               C.byref(self.tc), L.ptr(self.loss), L.stream_of())
        self.ws.n_rays = n
        self.ws.generation += 1
        return self.loss

    # ------------------------------------------------------- checkpoints
    def save_checkpoint(self, prefix: str, global_step: int = 0) -> str:
        """Everything a resumed run needs, as run.py:612-630 + VDBAdam.save_to
        (masked_adam.py:82-95) lay it out beside ``prefix`` (e.g. ``<dir>/fine``):
        ``<prefix>_last.npz`` (model kwargs, rgbnet parameters, Adam moments and
        scalars, the voxel optimisers' scalars, global_step),
        ``<prefix>density.pvdb`` / ``<prefix>color.pvdb`` (the grids) and
        ``<prefix>density_exp_avg.vdb`` ... (the voxel-Adam moments). Returns
        the path of the ``_last.npz`` file."""
        torch.cuda.synchronize()
        cfg = self.cfg
        path = prefix + "_last.npz"
        scal = {}
        for tag, o in (("d", self.dopt), ("c", self.kopt)):
            scal.update({tag + "step": o.getStep(), tag + "lr": o.getLr(), tag + "eps": o.getEps(),
                         tag + "beta0": o.getBeta0(), tag + "beta1": o.getBeta1()})
        np.savez(path, global_step=np.int64(global_step),
                 xyz_min=np.array(cfg.xyz_min, np.float32),
                 xyz_max=np.array(cfg.xyz_max, np.float32),
                 act_shift=np.float32(cfg.act_shift), voxel_size_ratio=np.float32(cfg.interval),
                 world_size=np.array(self.density.reso, np.int32),
                 params=self.params.cpu().numpy(), exp_avg=self.exp_avg.cpu().numpy(),
                 exp_avg_sq=self.exp_avg_sq.cpu().numpy(), rgbnet_step=np.int32(self._step.value),
                 rgbnet_lr=np.float32(self._lr.value),
                 **{k: np.asarray(v) for k, v in scal.items()})
        self.density.save_to(prefix + "density.pvdb")
        self.k0.save_to(prefix + "color.pvdb")
        self.dopt.save_to(prefix + "density_")
        self.kopt.save_to(prefix + "color_")
        return path

    def load_checkpoint(self, prefix: str) -> int:
        """Restores a checkpoint written by save_checkpoint into this trainer
        (same grid topology and rgbnet shape; values are copied in place, so the
        captured step graph stays valid). Returns the saved global_step."""
        st = np.load(prefix + "_last.npz")
        if st["params"].size != self.params.numel():
            raise ValueError("the checkpoint's rgbnet has another shape")
        self.density.load_from(prefix + "density.pvdb")
        self.k0.load_from(prefix + "color.pvdb")
        self.dopt.load_from(prefix + "density_")
        self.kopt.load_from(prefix + "color_")
        for tag, o in (("d", self.dopt), ("c", self.kopt)):
            o.setStep(int(st[tag + "step"]))
            o.setLr(float(st[tag + "lr"]))
            o.setEps(float(st[tag + "eps"]))
            o.setBeta0(float(st[tag + "beta0"]))
            o.setBeta1(float(st[tag + "beta1"]))
        for t, key in ((self.params, "params"), (self.exp_avg, "exp_avg"),
                       (self.exp_avg_sq, "exp_avg_sq")):
            t.copy_(torch.from_numpy(st[key]).to(t.device))
        self._step.value = int(st["rgbnet_step"])
        self._lr.value = float(st["rgbnet_lr"])
        # gradients restart clean, as after a step
        self.density.zero_grad()
        self.k0.zero_grad()
        self.grads.zero_()
        torch.cuda.synchronize()
        return int(st["global_step"])
