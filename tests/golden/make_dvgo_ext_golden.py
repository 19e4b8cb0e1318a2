"""Writes tests/golden/dvgo_ext_golden.npz: golden vectors from the
reference's own DirectVoxGO torch extensions, run on a GPU.

The extensions are the reference's lib/cuda/render_utils_kernel.cu,
total_variation_kernel.cu and adam_upd_kernel.cu (with their .cpp bindings),
staged unmodified into oracle/_ref/dvgo_ext/ by oracle/build.py where the
reference tree is mounted, and JIT-compiled here for sm_103a by
oracle.build.load_dvgo_ext. The inputs are seeded and stored in the fixture
beside the outputs, so the tests need neither the reference nor a GPU to read
them:

* sample_pts_on_rays (render_utils_kernel.cu:196-242): ragged camera rays,
  rays that miss the bbox, axis-aligned rays (zero direction components),
  rays starting inside the bbox, grazing rays with a single sample;
* maskcache_lookup (:373-424): points inside and outside the mask volume and
  on rounding boundaries;
* raw2alpha / raw2alpha_backward (:430-443, :506-517) at intervals 0.5 and 1,
  including overflowing and vanishing exponentials;
* alpha2weight / alpha2weight_backward (:576-707): ragged rays with no,
  one and many samples, rays that stop at T < 1e-3 and rays that do not;
* total_variation_add_grad (total_variation_kernel.cu:13-67): 1 and 12
  channels, dense and sparse (grad != 0) modes;
* adam_upd, masked_adam_upd, adam_upd_with_perlr (adam_upd_kernel.cu:8-132):
  three steps each, gradients with zeros.

Usage (on a machine with a GPU, after oracle/build.py staged the sources):
    python tests/golden/make_dvgo_ext_golden.py [out.npz]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

XYZ_MIN = np.array([-1.5, -1.5, -1.5], np.float32)
XYZ_MAX = np.array([1.5, 1.5, 1.5], np.float32)
NEAR, FAR = 2.0, 1e9
STEPDIST = 0.5 * 3.0 / 160  # half a voxel of the 160^3 grid, world units
ACT_SHIFT = float(np.float32(np.log(1 / (1 - 1e-2) - 1)))  # dvgo.py:48, alpha_init 1e-2


def make_rays(rng):
    """Seeded rays of every kind the sampler distinguishes."""
    def sphere(n, r=4.03):
        v = rng.normal(size=(n, 3))
        return (v / np.linalg.norm(v, axis=1, keepdims=True) * r).astype(np.float32)

    o_hit = sphere(160)
    tgt = rng.uniform(-1.2, 1.2, (160, 3))
    d_hit = (tgt - o_hit) * rng.uniform(0.2, 1.5, (160, 1))  # unnormalised, like get_rays
    o_miss = sphere(16)
    d_miss = o_miss * rng.uniform(0.1, 1.0, (16, 1)) + rng.normal(0, 0.1, (16, 3))  # away
    o_axis = np.array([[0.3, 0.2, 4.03], [-0.7, 4.03, 0.1], [4.03, 0.0, 0.0], [0.0, 0.0, -4.03],
                       [1.0, -1.0, 4.0], [3.0, 0.5, -0.5]], np.float32)
    d_axis = np.array([[0, 0, -1], [0, -1, 0], [-1, 0, 0], [0, 0, 1], [0, 0, -2], [-1, 0, 0]],
                      np.float32)
    o_in = rng.uniform(-1.0, 1.0, (8, 3))
    d_in = rng.normal(size=(8, 3))
    # grazing rays through a bbox corner region: 1-2 samples
    o_gr = np.tile(np.array([[4.03, 4.03, 4.03]], np.float32), (6, 1))
    d_gr = (np.array([[1.5, 1.5, 1.5]]) + rng.normal(0, 0.004, (6, 3))) - o_gr
    ro = np.concatenate([o_hit, o_miss, o_axis, o_in, o_gr]).astype(np.float32)
    rd = np.concatenate([d_hit, d_miss, d_axis, d_in, d_gr]).astype(np.float32)
    return ro, rd


def main(out_path: str) -> None:
    import torch
    from oracle import build as ob

    assert torch.cuda.is_available(), "the reference extensions need a GPU"
    ru = ob.load_dvgo_ext("render_utils_cuda")
    tvx = ob.load_dvgo_ext("total_variation_cuda")
    adx = ob.load_dvgo_ext("adam_upd_cuda")
    dev = "cuda"
    rng = np.random.default_rng(20261204)
    G = {}

    def T(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    def N(t):
        return t.detach().cpu().numpy()

    # ---- sample_pts_on_rays
    ro, rd = make_rays(rng)
    res = ru.sample_pts_on_rays(T(ro), T(rd), T(XYZ_MIN), T(XYZ_MAX), NEAR, FAR, STEPDIST)
    pts, ob_, rid, sid, nst, tmin, tmax = (N(x) for x in res)
    G.update(sp_rays_o=ro, sp_rays_d=rd, sp_xyz_min=XYZ_MIN, sp_xyz_max=XYZ_MAX,
             sp_params=np.array([NEAR, FAR, STEPDIST], np.float64),
             sp_pts=pts.astype(np.float32), sp_mask_outbbox=ob_.astype(np.uint8),
             sp_ray_id=rid.astype(np.int32), sp_step_id=sid.astype(np.int32),
             sp_n_steps=nst.astype(np.int64), sp_t_min=tmin, sp_t_max=tmax)

    # ---- maskcache_lookup
    world = rng.random((37, 40, 29)) < 0.35
    xyz = rng.uniform(-1.8, 1.8, (6000, 3)).astype(np.float32)
    xyz[:400] = (np.round(xyz[:400] * 20) / 20).astype(np.float32)  # near .5 boundaries
    scale = ((np.array(world.shape) - 1) / (XYZ_MAX - XYZ_MIN)).astype(np.float32)
    shift = (-XYZ_MIN * scale).astype(np.float32)
    mc = N(ru.maskcache_lookup(T(world), T(xyz), T(scale), T(shift)))
    G.update(mc_world=np.packbits(world.reshape(-1)), mc_shape=np.array(world.shape, np.int32),
             mc_xyz=xyz, mc_scale=scale, mc_shift=shift, mc_out=mc.astype(np.uint8))

    # ---- raw2alpha (+ backward)
    dens = rng.normal(0, 4, 20000).astype(np.float32)
    dens[:10] = [-200.0, -60.0, -20.0, 0.0, 4.595, 20.0, 60.0, 88.0, 95.0, 300.0]
    for tag, interval in (("05", 0.5), ("10", 1.0)):
        e, a = ru.raw2alpha(T(dens), ACT_SHIFT, interval)
        gb = rng.normal(0, 1, dens.size).astype(np.float32)
        gd = ru.raw2alpha_backward(e, T(gb), interval)
        G.update({f"ra{tag}_grad_back": gb, f"ra{tag}_exp": N(e), f"ra{tag}_alpha": N(a),
                  f"ra{tag}_grad": N(gd)})
    G.update(ra_density=dens, ra_params=np.array([ACT_SHIFT, 0.5, 1.0], np.float64))

    # ---- alpha2weight (+ backward)
    n_rays = 400
    counts = rng.integers(0, 500, n_rays)
    counts[:6] = [0, 1, 0, 2, 1, 0]
    counts[-1] = 3
    ray_id = np.repeat(np.arange(n_rays), counts).astype(np.int64)
    alpha = (rng.random(ray_id.size) ** 6 * 0.2).astype(np.float32)
    heavy = rng.random(n_rays) < 0.4  # rays that reach T < 1e-3
    alpha[heavy[ray_id]] = rng.beta(0.8, 1.5, int(heavy[ray_id].sum())).astype(np.float32)
    alpha[::53] = 0.999
    w, Tt, last, i_s, i_e = ru.alpha2weight(T(alpha), T(ray_id), n_rays)
    gw = rng.normal(0, 1, ray_id.size).astype(np.float32)
    gl = rng.normal(0, 1, n_rays).astype(np.float32)
    ga = ru.alpha2weight_backward(T(alpha), w, Tt, last, i_s, i_e, n_rays, T(gw), T(gl))
    G.update(aw_alpha=alpha, aw_ray_id=ray_id.astype(np.int32), aw_n_rays=np.int64(n_rays),
             aw_weight=N(w), aw_T=N(Tt), aw_last=N(last), aw_i_start=N(i_s), aw_i_end=N(i_e),
             aw_grad_weights=gw, aw_grad_last=gl, aw_grad=N(ga))

    # ---- total_variation_add_grad on dense [1, C, X, Y, Z] grids
    shape = (21, 18, 16)
    for tag, C, wxyz, dense in (("c1d", 1, (0.3, 0.3, 0.3), True),
                                ("c1s", 1, (0.25, 0.25, 0.25), False),
                                ("c12s", 12, (0.2, 0.2, 0.2), False),
                                ("c12d", 12, (0.4, 0.1, 0.4), True)):
        p = rng.normal(0, 0.7, (1, C) + shape).astype(np.float32)
        g = rng.normal(0, 1, p.shape).astype(np.float32)
        g[rng.random(p.shape) < 0.6] = 0.0
        gt = T(g).clone()
        tvx.total_variation_add_grad(T(p), gt, wxyz[0], wxyz[1], wxyz[2], dense)
        G.update({f"tv{tag}_param": p, f"tv{tag}_grad_in": g, f"tv{tag}_grad_out": N(gt),
                  f"tv{tag}_w": np.array(wxyz, np.float32), f"tv{tag}_dense": np.int64(dense)})

    # ---- dense Adam, three modes, three steps each
    n = 6000
    lr, b1, b2, eps = 1e-3, 0.9, 0.99, 1e-8
    for mode in (0, 1, 2):
        p = T(rng.normal(0, 0.5, n).astype(np.float32))
        m = torch.zeros_like(p)
        v = torch.zeros_like(p)
        perlr = T(rng.random(n).astype(np.float32))
        G[f"adam{mode}_p0"] = N(p)
        G[f"adam{mode}_perlr"] = N(perlr)
        for step in (1, 2, 3):
            g = rng.normal(0, 1, n).astype(np.float32)
            g[rng.random(n) < 0.3] = 0.0
            if mode == 0:
                adx.adam_upd(p, T(g), m, v, step, b1, b2, lr, eps)
            elif mode == 1:
                adx.masked_adam_upd(p, T(g), m, v, step, b1, b2, lr, eps)
            else:
                adx.adam_upd_with_perlr(p, T(g), m, v, perlr, step, b1, b2, lr, eps)
            G.update({f"adam{mode}_g{step}": g, f"adam{mode}_p{step}": N(p),
                      f"adam{mode}_m{step}": N(m), f"adam{mode}_v{step}": N(v)})
    G["adam_params"] = np.array([lr, b1, b2, eps], np.float64)
    torch.cuda.synchronize()
    G["torch_version"] = np.array(torch.__version__)
    np.savez_compressed(out_path, **G)
    print(f"wrote {out_path}: {len(G)} arrays, {os.path.getsize(out_path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.path.join(ROOT, "tests", "golden", "dvgo_ext_golden.npz"))
