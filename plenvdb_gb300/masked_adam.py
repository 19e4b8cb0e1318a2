"""Optimisers with the reference's interface (plenvdb/lib/masked_adam.py).

* ``VDBAdam`` (masked_adam.py:18-95): per-voxel Adam over a density and a k0
  VDB grid, modes 0 (plain) / 1 (skip zero gradients) / 2 (per-voxel lr).
* ``MaskedAdam`` (masked_adam.py:105-158): dense Adam for torch parameters
  (the rgbnet), through libpvdb's pvdb_adam_dense kernel.
"""
from __future__ import annotations

import os

import torch

from . import _lib as L
from .plenvdb import ColorOpt, DensityOpt


def _check_hparams(lr, betas, eps):
    """The value checks both optimisers make on construction (masked_adam.py:20-27,
    :103-110): non-negative lr and eps, betas in [0, 1). ValueError names the
    offending value."""
    bad = [(not 0.0 <= lr, f"Invalid learning rate: {lr}"),
           (not 0.0 <= eps, f"Invalid epsilon value: {eps}")]
    bad += [(not 0.0 <= b < 1.0, f"Invalid beta parameter at index {i}: {b}")
            for i, b in enumerate(betas[:2])]
    for failed, msg in bad:
        if failed:
            raise ValueError(msg)


class VDBAdam:
    """Per-voxel Adam over the two VDB grids (density and k0); `params` holds
    one group per grid: {"params": VDBGrid-like (channels, grid), "lr": float,
    "skip_zero_grad": bool}."""

    def __init__(self, params, lr=1e-3, betas=(0.9, 0.99), eps=1e-8):
        _check_hparams(lr, betas, eps)
        assert len(params) == 2
        self.has_per_lr = False
        b0, b1 = betas[0], betas[1]
        by_kind = {("density" if g["params"].channels == 1 else "color"): g for g in params}
        dgrp, cgrp = by_kind["density"], by_kind["color"]
        self.densityparam, self.colorparam = dgrp["params"], cgrp["params"]
        self.densityOpt = DensityOpt(self.densityparam.grid, dgrp["lr"], eps, b0, b1)
        self.colorOpt = ColorOpt(self.colorparam.grid, cgrp["lr"], eps, b0, b1)
        self.skip_density = dgrp["skip_zero_grad"]
        self.skip_color = cgrp["skip_zero_grad"]

    def set_pervoxel_lr(self, count):
        self.has_per_lr = True
        per_lr = (count.float() / count.max()).reshape(-1)
        self.densityOpt.set_pervoxel_lr(per_lr if per_lr.is_cuda else per_lr.numpy())

    def update_lr(self, factor):
        self.densityOpt.update_lr(factor)
        self.colorOpt.update_lr(factor)

    def zero_grad(self):
        self.densityOpt.zero_grad()
        self.colorOpt.zero_grad()

    def step(self):
        # stepmode: 0 default, 1 skip zero grad, 2 per-voxel lr (masked_adam.py:56-68)
        if self.has_per_lr:
            self.densityOpt.step(2)
        elif self.skip_density:
            self.densityOpt.step(1)
        else:
            self.densityOpt.step(0)
        self.colorOpt.step(1 if self.skip_color else 0)

    def state_scalars(self):
        d, c = self.densityOpt, self.colorOpt
        return {"dlr": d.getLr(), "clr": c.getLr(), "deps": d.getEps(), "ceps": c.getEps(),
                "dbeta0": d.getBeta0(), "cbeta0": c.getBeta0(), "dbeta1": d.getBeta1(),
                "cbeta1": c.getBeta1(), "dstep": d.getStep(), "cstep": c.getStep()}

    def load_from(self, loadpath):
        ckpt = torch.load(loadpath + "vdbopt.tar")
        d, c = self.densityOpt, self.colorOpt
        d.setStep(ckpt["dstep"]); d.setLr(ckpt["dlr"]); d.setBeta0(ckpt["dbeta0"])
        d.setBeta1(ckpt["dbeta1"]); d.setEps(ckpt["deps"])
        c.setStep(ckpt["cstep"]); c.setLr(ckpt["clr"]); c.setBeta0(ckpt["cbeta0"])
        c.setBeta1(ckpt["cbeta1"]); c.setEps(ckpt["ceps"])
        d.load_from(loadpath + "density_")
        c.load_from(loadpath + "color_")

    def save_to(self, savepath):
        torch.save(self.state_scalars(), savepath + "vdbopt.tar")
        self.densityOpt.save_to(savepath + "density_")
        self.colorOpt.save_to(savepath + "color_")


class MaskedAdam(torch.optim.Optimizer):
    """Dense Adam over torch parameters (the rgbnet), with the reference's
    skip-zero-gradient and per-voxel learning-rate modes."""

    def __init__(self, params, lr=1e-3, betas=(0.9, 0.99), eps=1e-8):
        _check_hparams(lr, betas, eps)
        self.per_lr = None
        super().__init__(params, {"lr": lr, "betas": betas, "eps": eps})

    def set_pervoxel_lr(self, count):
        assert self.param_groups[0]["params"][0].shape == count.shape
        self.per_lr = count.float() / count.max()

    @torch.no_grad()
    def step(self):
        for group in self.param_groups:
            lr = group["lr"]
            beta1, beta2 = group["betas"]
            eps = group["eps"]
            skip_zero_grad = group.get("skip_zero_grad", False)
            for param in group["params"]:
                if param.grad is None:
                    continue
                if param.dtype != torch.float32 or not param.is_cuda or not param.is_contiguous():
                    raise ValueError("MaskedAdam needs contiguous CUDA float32 parameters")
                state = self.state[param]
                if len(state) == 0:
                    state["step"] = 0
                    state["exp_avg"] = torch.zeros_like(param, memory_format=torch.preserve_format)
                    state["exp_avg_sq"] = torch.zeros_like(param,
                                                           memory_format=torch.preserve_format)
                state["step"] += 1
                grad = param.grad.contiguous()
                if self.per_lr is not None and param.shape == self.per_lr.shape:
                    mode, perlr = 2, self.per_lr.contiguous()
                elif skip_zero_grad:
                    mode, perlr = 1, None
                else:
                    mode, perlr = 0, None
                L.call("pvdb_adam_dense", L.ptr(param), L.ptr(grad), L.ptr(state["exp_avg"]),
                       L.ptr(state["exp_avg_sq"]), L.ptr(perlr), param.numel(), state["step"],
                       float(beta1), float(beta2), float(lr), float(eps), mode, L.stream_of())
