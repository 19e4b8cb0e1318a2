"""Generates tests/golden/lifecycle_golden.npz by running the reference's own
Python code for the DVGO schedule around the training step:

* lib/dvgo.py  get_rays / ndc_rays / get_rays_of_a_view, batch_indices_generator,
               DirectVoxGO.update_occupancy_cache, .scale_volume_grid (the
               mask-cache rebuild), .maskout_near_cam_vox, .voxel_count_views
* lib/grid.py  VDBGrid.wld2idx, VDBGrid.scale_volume_grid, MaskGrid, DenseGrid
* vdb_compression.py (run as a script)

The reference modules load CUDA extensions and OpenVDB when imported, so the
functions are taken out of the source with `ast` and executed with stand-ins
for what they call outside Python: the VDB classes (plain array holders), the
two render_utils_cuda kernels the occupancy code needs (raw2alpha and
maskcache_lookup, from the oracle's restatement, itself checked against the
CUDA kernels by tests/test_gpu_render_utils.py), DensityVDB's trilinear
forward (the oracle's FP32 restatement, pinned by nanovdb_golden.npz) and
pyopenvdb (a reader/writer of in-memory arrays).

Run where the reference tree is mounted:

    python tests/golden/make_lifecycle_golden.py
"""
from __future__ import annotations

import argparse
import ast
import os
import shutil
import sys
import tempfile
import textwrap
import types

import numpy as np
import torch
import torch.nn as nn
import torch.nn.functional as F

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# the reference tree: $PVDB_REFERENCE_ROOT (default /root/reference)
REF = os.path.join(os.environ.get("PVDB_REFERENCE_ROOT", "/root/reference"), "plenvdb")
OUT = os.path.join(HERE, "lifecycle_golden.npz")


def _source(path, name, cls=None):
    src = open(path).read()
    tree = ast.parse(src)
    body = tree.body
    if cls is not None:
        body = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls).body
    node = next(n for n in body if isinstance(n, (ast.FunctionDef, ast.ClassDef)) and n.name == name)
    return textwrap.dedent(ast.get_source_segment(src, node))


def _load(path, name, cls=None, extra=None):
    ns = {"torch": torch, "nn": nn, "F": F, "np": np, "time": __import__("time")}
    ns.update(extra or {})
    exec(compile(_source(path, name, cls), f"{path}:{name}", "exec"), ns)
    return ns[name]


DVGO = os.path.join(REF, "lib", "dvgo.py")
GRID = os.path.join(REF, "lib", "grid.py")


def _oracle_grid(dense, background=0.0):
    R = dense.shape
    return O.OGridData(R, dense.astype(np.float64), np.ones(R, np.uint8), background=background)


class _RenderUtils:
    """The two render_utils_cuda kernels the occupancy code calls."""

    @staticmethod
    def maskcache_lookup(world, xyz, scale, shift):
        out = O.maskcache(world.numpy().astype(np.uint8), xyz.numpy(), scale.numpy(),
                          shift.numpy())
        return torch.from_numpy(out)


class _Raw2Alpha:
    @staticmethod
    def apply(density, shift, interval):
        e, a = O.raw2alpha(density.detach().numpy().astype(np.float32), float(shift),
                           float(interval), fp32=True)
        return torch.from_numpy(a.astype(np.float32))


def rays_cases(out):
    ns = {}
    get_rays = _load(DVGO, "get_rays")
    ndc_rays = _load(DVGO, "ndc_rays")
    view = _load(DVGO, "get_rays_of_a_view", extra={"get_rays": get_rays, "ndc_rays": ndc_rays})
    ns["get_rays"] = get_rays
    rng = np.random.default_rng(1)
    H, W = 12, 10
    K = np.array([[11.3, 0, 4.9], [0, 12.7, 6.1], [0, 0, 1]], np.float64)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    c2w = np.eye(4, dtype=np.float32)
    c2w[:3, :3] = q.astype(np.float32)
    c2w[:3, 3] = np.array([0.3, -1.2, 3.9], np.float32)
    c2w_t = torch.from_numpy(c2w)
    cases = [("center", False, False, False, False), ("lefttop", True, True, False, False),
             ("center", False, True, True, False), ("center", False, False, False, True),
             ("random", False, True, True, False)]
    out["rays_K"] = K
    out["rays_c2w"] = c2w
    out["rays_HW"] = np.array([H, W])
    for n, (mode, inv, fx, fy, ndc) in enumerate(cases):
        torch.manual_seed(100 + n)
        o, d, v = view(H, W, K, c2w_t, ndc, inv, fx, fy, mode=mode)
        out[f"rays{n}_flags"] = np.array([["center", "lefttop", "random"].index(mode), inv, fx,
                                          fy, ndc, 100 + n])
        out[f"rays{n}_o"] = o.numpy()
        out[f"rays{n}_d"] = d.numpy()
        out[f"rays{n}_v"] = v.numpy()
    out["rays_ncases"] = np.array(len(cases))


def batches_case(out):
    gen_fn = _load(DVGO, "batch_indices_generator")
    np.random.seed(7)
    g = gen_fn(50, 16)
    out["batches"] = np.stack([next(g).numpy() for _ in range(8)])


def compression_case(out):
    rng = np.random.default_rng(2)
    R = (9, 7, 11)
    mask = rng.random(R) < 0.3
    den = rng.normal(0, 3, R).astype(np.float32)
    col = rng.normal(0, 0.2, R + (12,)).astype(np.float32)
    col[0, 0, 0, 0] = 70000.0  # overflows FP16
    col[1, 1, 1, 1] = 1e-8     # FP16 subnormal range
    captured = {}

    class Tree:
        def __init__(self, arr=None):
            self.arr = arr

        def copyToArray(self, arr):
            arr[...] = self.arr

        def copyFromArray(self, arr):
            captured["idxs"] = np.array(arr)

    vdb = types.ModuleType("pyopenvdb")
    vdb.FloatGrid = Tree

    def readAll(path):
        if path.endswith("finedensity.vdb"):
            return ([Tree(den.astype(np.float64))],)
        return ([Tree(col[..., 3 * i:3 * i + 3].astype(np.float64)) for i in range(4)],)

    vdb.readAll = readAll
    vdb.write = lambda path, grids: None
    work = tempfile.mkdtemp(prefix="compression_", dir=HERE)  # removed below
    os.makedirs(os.path.join(work, "vdb_synth"), exist_ok=True)
    argv, tload = sys.argv, torch.load
    try:
        sys.modules["pyopenvdb"] = vdb
        sys.argv = ["vdb_compression.py", "--basedir", work, "--scenes", "synth"]
        torch.load = lambda path: {"model_state_dict": {"mask_cache.mask": torch.from_numpy(mask)}}
        path = os.path.join(REF, "vdb_compression.py")
        exec(compile(open(path).read(), path, "exec"), {"__name__": "__main__"})
    finally:
        sys.argv, torch.load = argv, tload
        sys.modules.pop("pyopenvdb", None)
    z = np.load(os.path.join(work, "vdb_synth", "mergeddata.npz"))
    out["merge_mask"] = mask
    out["merge_den"] = den
    out["merge_col"] = col
    out["merge_idxs"] = captured["idxs"]
    out["merge_den_rows"] = z["den"]
    out["merge_col_rows"] = z["col"]
    shutil.rmtree(work)


def scale_case(out):
    captured = {}

    class VDB:
        def __init__(self, reso, n):
            self.n = n

        def resetTimer(self):
            pass

        def copyFromDense(self, arr):
            captured["arr"] = np.array(arr)

    fn = _load(GRID, "scale_volume_grid", cls="VDBGrid",
               extra={"DensityVDB": VDB, "ColorVDB": VDB})
    rng = np.random.default_rng(3)
    for n, (src, dst, C) in enumerate([((6, 5, 7), (11, 9, 13), 1), ((9, 8, 6), (5, 12, 6), 12)]):
        vals = rng.normal(0, 1, src + (C,)).astype(np.float32)
        self = types.SimpleNamespace(channels=C)
        t = torch.from_numpy(vals).permute(3, 0, 1, 2).unsqueeze(0).contiguous()
        self.get_dense_grid = lambda t=t: t
        fn(self, torch.tensor(dst))
        out[f"scale{n}_src"] = vals
        out[f"scale{n}_dst"] = np.array(dst)
        out[f"scale{n}_out"] = captured["arr"].reshape(dst + (C,))


def occupancy_cases(out):
    rng = np.random.default_rng(4)
    R = (12, 10, 14)
    xyz_min = np.array([-1.5, -1.2, -1.4], np.float32)
    xyz_max = np.array([1.5, 1.3, 1.1], np.float32)
    dens = rng.normal(-2.0, 3.0, R).astype(np.float32)
    shift, interval, thres = -4.6, 0.5, 1e-3
    g = _oracle_grid(dens)
    wld2idx = _load(GRID, "wld2idx", cls="VDBGrid")
    vg = types.SimpleNamespace(xyz_min=torch.from_numpy(xyz_min), xyz_max=torch.from_numpy(xyz_max),
                               world_size=torch.tensor(R))

    def density(xyz):
        shape = xyz.shape[:-1]
        idx = wld2idx(vg, xyz.reshape(-1, 3)).numpy().astype(np.float32)
        return torch.from_numpy(O.sample(g, idx, fp32=True)[:, 0].astype(np.float32)).reshape(shape)

    def activate_density(d, interval=interval):
        return _Raw2Alpha.apply(d.flatten(), shift, interval).reshape(d.shape)

    MaskGrid = _load(GRID, "MaskGrid", extra={"render_utils_cuda": _RenderUtils})
    old = rng.random((9, 8, 10)) < 0.6
    # mode 0: update_occupancy_cache
    upd = _load(DVGO, "update_occupancy_cache", cls="DirectVoxGO")
    mc = MaskGrid(path=None, mask=torch.from_numpy(old.copy()), xyz_min=xyz_min, xyz_max=xyz_max)
    self = types.SimpleNamespace(xyz_min=torch.from_numpy(xyz_min),
                                 xyz_max=torch.from_numpy(xyz_max), mask_cache=mc,
                                 density=density, activate_density=activate_density,
                                 fast_color_thres=thres)
    upd(self)
    out["occ_dens"] = dens
    out["occ_box"] = np.stack([xyz_min, xyz_max])
    out["occ_params"] = np.array([shift, interval, thres], np.float32)
    out["occ_old"] = old
    out["occ_mode0"] = self.mask_cache.mask.numpy()
    # mode 1: DirectVoxGO.scale_volume_grid's rebuild (the grids were rescaled
    # already: density.get_dense_grid gives the new values)
    svg = _load(DVGO, "scale_volume_grid", cls="DirectVoxGO", extra={"grid": types.SimpleNamespace(MaskGrid=MaskGrid)})
    mc = MaskGrid(path=None, mask=torch.from_numpy(old.copy()), xyz_min=xyz_min, xyz_max=xyz_max)
    dgrid = types.SimpleNamespace(scale_volume_grid=lambda ws: None,
                                  get_dense_grid=lambda: torch.from_numpy(dens)[None, None])
    self = types.SimpleNamespace(world_size=torch.tensor(R), xyz_min=torch.from_numpy(xyz_min),
                                 xyz_max=torch.from_numpy(xyz_max), mask_cache=mc,
                                 density=dgrid, k0=dgrid, activate_density=activate_density,
                                 fast_color_thres=thres, _set_grid_resolution=lambda n: None)
    svg(self, int(np.prod(R)))
    out["occ_mode1"] = self.mask_cache.mask.numpy()
    # mode 2: MaskGrid(path=...) from a checkpoint's density
    st = {"model_state_dict": {"act_shift": torch.tensor(shift)},
          "model_kwargs": {"mask_cache_world_size": list(R), "voxel_size_ratio": interval,
                           "xyz_min": xyz_min.tolist(), "xyz_max": xyz_max.tolist()}}

    class DVDB:
        def __init__(self, reso, n):
            pass

        def load_from(self, path):
            pass

        def get_dense_grid(self):
            return dens.reshape(-1)

    tload = torch.load
    try:
        torch.load = lambda path: st
        MG2 = _load(GRID, "MaskGrid", extra={"render_utils_cuda": _RenderUtils,
                                             "DensityVDB": DVDB})
        m2 = MG2(path="ckpt/coarse_last.tar", mask_cache_thres=thres)
    finally:
        torch.load = tload
    out["occ_mode2"] = m2.mask.numpy()


def near_cam_case(out):
    rng = np.random.default_rng(5)
    R = (10, 12, 9)
    xyz_min = np.array([-1.0, -1.5, -1.2], np.float32)
    xyz_max = np.array([1.4, 1.5, 1.3], np.float32)
    cams = rng.uniform(-1.3, 1.3, (7, 3)).astype(np.float32)
    captured = {}
    dens = types.SimpleNamespace(
        setValuesOn_bymask=lambda m, v: captured.update(mask=m.numpy().copy(), val=v))
    fn = _load(DVGO, "maskout_near_cam_vox", cls="DirectVoxGO")
    self = types.SimpleNamespace(xyz_min=torch.from_numpy(xyz_min),
                                 xyz_max=torch.from_numpy(xyz_max), world_size=torch.tensor(R),
                                 density=dens)
    fn(self, torch.from_numpy(cams), 0.55)
    out["near_box"] = np.stack([xyz_min, xyz_max])
    out["near_cams"] = cams
    out["near_clip"] = np.array(0.55, np.float32)
    out["near_mask"] = captured["mask"].reshape(R)


def count_views_case(out):
    DenseGrid = _load(GRID, "DenseGrid")
    fn = _load(DVGO, "voxel_count_views", cls="DirectVoxGO",
               extra={"grid": types.SimpleNamespace(DenseGrid=DenseGrid)})
    rng = np.random.default_rng(6)
    R = (14, 12, 16)
    xyz_min = np.array([-1.5, -1.5, -1.5], np.float32)
    xyz_max = np.array([1.5, 1.5, 1.5], np.float32)
    voxel_size = np.float32(3.0 / 14)
    n_views, H, W = 3, 6, 5
    ro = np.zeros((n_views, H, W, 3), np.float32)
    rd = np.zeros((n_views, H, W, 3), np.float32)
    for v in range(n_views):
        c = rng.normal(size=3)
        c = (3.5 * c / np.linalg.norm(c)).astype(np.float32)
        ro[v] = c
        tgt = rng.uniform(-0.8, 0.8, (H, W, 3)).astype(np.float32)
        rd[v] = tgt - c
    rd[0, 0, 0] = [0.0, 0.0, -1.0]  # a zero component (the 1e-6 substitute)
    ro[0, 0, 0] = [0.1, -0.2, 3.0]
    self = types.SimpleNamespace(world_size=torch.tensor(R), xyz_min=torch.from_numpy(xyz_min),
                                 xyz_max=torch.from_numpy(xyz_max),
                                 voxel_size=torch.tensor(voxel_size),
                                 density=types.SimpleNamespace(
                                     get_dense_grid=lambda: torch.zeros([1, 1, *R])))
    cnt = fn(self, torch.from_numpy(ro), torch.from_numpy(rd), [1] * n_views, 0.5, 6.0, 0.5)
    out["cv_ro"] = ro
    out["cv_rd"] = rd
    out["cv_box"] = np.stack([xyz_min, xyz_max])
    out["cv_params"] = np.array([voxel_size, 0.5, 0.5], np.float32)  # voxel_size, near, stepsize
    out["cv_reso"] = np.array(R)
    out["cv_count"] = cnt.detach().numpy()


def main():
    if not os.path.isdir(REF):
        raise SystemExit("reference tree not mounted: cannot run the reference functions")
    out = {}
    rays_cases(out)
    batches_case(out)
    compression_case(out)
    scale_case(out)
    occupancy_cases(out)
    near_cam_case(out)
    count_views_case(out)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {len(out)} arrays, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    argparse.ArgumentParser(description=__doc__).parse_args()
    main()
