"""Generates tests/golden/nanovdb_golden.npz from the reference's own NanoVDB.

Run where the reference tree is mounted (it builds oracle/_ref/libnanoref.so
from oracle/ref_harness.cpp, which includes nanovdb/NanoVDB.h and
nanovdb/util/GridBuilder.h from the reference):

    python tests/golden/make_golden.py

The fixture pins the CPU oracle (oracle/pvdb_oracle.cpp) to the reference's
leaf/voxel lookup rules, trilinear sampling, gradient scatter, voxel Adam and
the merged-index density of the renderer (see oracle/ref_harness.cpp for the
reference lines each entry point restates).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nanovdb_golden.npz")


def p(a):
    return C.c_void_p(a.ctypes.data)


def main():
    path = obuild.build_ref()
    if path is None:
        raise SystemExit("reference tree not mounted: cannot build the NanoVDB harness")
    lib = C.CDLL(path)
    for n in ("nref_build_float", "nref_build_vec3"):
        getattr(lib, n).restype = C.c_void_p
    rng = np.random.default_rng(20231203)

    # ---- topology: R=20 (partial last leaf), sparse active set, background -10
    R = 20
    P = 24
    reso = np.array([R, R, R], np.int32)
    pad = np.array([P, P, P], np.int32)
    active = np.zeros((P, P, P), np.uint8)
    active[:R, :R, :R] = (rng.random((R, R, R)) < 0.35).astype(np.uint8)
    active[:8, 16:, :] = 0          # a whole unallocated leaf column
    L = P // 8
    alloc = active.reshape(L, 8, L, 8, L, 8).max(axis=(1, 3, 5)).astype(np.uint8)
    dens = rng.normal(0, 1, (P, P, P)).astype(np.float32)
    k0 = rng.normal(0, 0.1, (P, P, P, 12)).astype(np.float32)
    bg = np.float32(-10.0)

    keep = []

    def fgrid(vals, bgv):
        vals = np.ascontiguousarray(vals, np.float32)
        keep.append(vals)
        return C.c_void_p(lib.nref_build_float(p(reso), p(pad), p(alloc), p(active), p(vals),
                                               C.c_float(bgv)))

    def vgrids(vals, bgv):
        vals = np.ascontiguousarray(vals, np.float32)
        keep.append(vals)
        return [C.c_void_p(lib.nref_build_vec3(p(reso), p(pad), p(alloc), p(active), p(vals), 4,
                                               d, C.c_float(bgv))) for d in range(4)]

    gd = fgrid(dens, bg)
    gk = vgrids(k0, 0.0)
    assert lib.nref_is_sequential(gd) == 1

    # ---- lookups, including negative and beyond-padding coordinates
    ijk = rng.integers(-4, P + 4, (3000, 3)).astype(np.int32)
    lk_val = np.empty(3000, np.float32)
    lk_act = np.empty(3000, np.uint8)
    lib.nref_lookup_float(gd, p(ijk), C.c_int64(3000), p(lk_val), p(lk_act))

    # ---- trilinear forward
    n = 3000
    xyz = rng.uniform(-1.5, R + 1.5, (n, 3)).astype(np.float32)
    xyz[:200] = np.floor(xyz[:200])  # exact lattice points
    xs, ys, zs = (np.ascontiguousarray(xyz[:, a]) for a in range(3))
    fwd_d = np.empty(n, np.float32)
    lib.nref_density_forward(gd, p(xs), p(ys), p(zs), C.c_int64(n), p(fwd_d))
    hs = (C.c_void_p * 4)(*gk)
    fwd_c = np.empty(n * 12, np.float32)
    lib.nref_color_forward(hs, 4, p(xs), p(ys), p(zs), C.c_int64(n), p(fwd_c))

    # ---- backward into zero grad grids (same topology)
    nb = 800
    bxyz = rng.uniform(-1.0, R + 0.5, (nb, 3)).astype(np.float32)
    bxs, bys, bzs = (np.ascontiguousarray(bxyz[:, a]) for a in range(3))
    gdens = rng.normal(0, 1, nb).astype(np.float32)
    gcol = rng.normal(0, 1, (nb, 12)).astype(np.float32)
    zero_f = np.zeros((P, P, P), np.float32)
    zero_v = np.zeros((P, P, P, 12), np.float32)
    gg = fgrid(zero_f, 0.0)
    lib.nref_density_backward(gg, p(bxs), p(bys), p(bzs), p(gdens), C.c_int64(nb))
    bwd_d = np.empty((R, R, R), np.float32)
    lib.nref_read_float(gg, p(reso), p(bwd_d))
    gkg = vgrids(zero_v, 0.0)
    hg = (C.c_void_p * 4)(*gkg)
    lib.nref_color_backward(hg, 4, p(bxs), p(bys), p(bzs), p(gcol), C.c_int64(nb))
    bwd_c = np.empty((R, R, R, 12), np.float32)
    lib.nref_read_vec3(hg, 4, p(reso), p(bwd_c))

    # ---- voxel Adam, modes 0/1/2, one step from random state
    grad_d = rng.normal(0, 1, (P, P, P)).astype(np.float32)
    grad_d[rng.random((P, P, P)) < 0.4] = 0.0
    m_d = rng.normal(0, 0.1, (P, P, P)).astype(np.float32)
    v_d = rng.uniform(0, 0.1, (P, P, P)).astype(np.float32)
    lr_d = rng.uniform(0.1, 1.0, (P, P, P)).astype(np.float32)
    grad_c = rng.normal(0, 1, (P, P, P, 12)).astype(np.float32)
    zmask = rng.random((P, P, P, 4)) < 0.4
    grad_c.reshape(P, P, P, 4, 3)[zmask] = 0.0
    grad_c.reshape(-1)[rng.random(grad_c.size) < 0.1] = 0.0  # partially zero Vec3 groups
    m_c = rng.normal(0, 0.1, (P, P, P, 12)).astype(np.float32)
    v_c = rng.uniform(0, 0.1, (P, P, P, 12)).astype(np.float32)
    stepsz, eps, b0, b1 = np.float32(0.0123), np.float32(1e-8), np.float32(0.9), np.float32(0.99)
    adam = {}
    for mode in (0, 1, 2):
        hd, hgr, hm, hv, hl = (fgrid(dens, bg), fgrid(grad_d, 0.0), fgrid(m_d, 0.0),
                               fgrid(v_d, 0.0), fgrid(lr_d, 0.0))
        lib.nref_density_adam(hd, hgr, hm, hv, hl if mode == 2 else None, C.c_float(stepsz),
                              C.c_float(eps), C.c_float(b0), C.c_float(b1), mode)
        for name, h in (("data", hd), ("m", hm), ("v", hv)):
            out = np.empty((R, R, R), np.float32)
            lib.nref_read_float(h, p(reso), p(out))
            adam[f"adam_d{mode}_{name}"] = out
        cd, cg, cm, cv = vgrids(k0, 0.0), vgrids(grad_c, 0.0), vgrids(m_c, 0.0), vgrids(v_c, 0.0)
        arr = lambda hs_: (C.c_void_p * 4)(*hs_)  # noqa: E731
        lib.nref_color_adam(arr(cd), arr(cg), arr(cm), arr(cv), hl if mode == 2 else None, 4,
                            C.c_float(stepsz), C.c_float(eps), C.c_float(b0), C.c_float(b1), mode)
        for name, h in (("data", cd), ("m", cm), ("v", cv)):
            out = np.empty((R, R, R, 12), np.float32)
            lib.nref_read_vec3(arr(h), 4, p(reso), p(out))
            adam[f"adam_c{mode}_{name}"] = out

    # ---- merged index grid (renderer): row ids as float values, row 0 = empty
    idx_act = active.copy()
    rows = np.zeros((P, P, P), np.float32)
    nrow = int(idx_act.sum())
    rows[idx_act > 0] = np.arange(1, nrow + 1, dtype=np.float32)
    den_rows = np.concatenate([[0.0], rng.normal(0, 2, nrow)]).astype(np.float32)
    hidx = C.c_void_p(lib.nref_build_float(p(reso), p(pad), p(alloc), p(idx_act), p(rows),
                                           C.c_float(0.0)))
    ni = 2000
    ixyz = rng.uniform(0.0, R - 1.0, (ni, 3)).astype(np.float32)
    ixyz[:100] = np.round(ixyz[:100]) + 0.5  # rint ties
    idx_den = np.empty(ni, np.float32)
    idx_act_round = np.empty(ni, np.uint8)
    lib.nref_index_density(hidx, p(den_rows), p(ixyz), C.c_int64(ni), p(idx_den),
                           p(idx_act_round))

    np.savez_compressed(
        OUT, reso=reso, active=active[:R, :R, :R], alloc=alloc, density=dens,
        k0=k0, background=bg, lookup_ijk=ijk, lookup_val=lk_val,
        lookup_active=lk_act, fwd_xyz=xyz, fwd_density=fwd_d, fwd_color=fwd_c.reshape(n, 12),
        bwd_xyz=bxyz, bwd_gdens=gdens, bwd_gcol=gcol, bwd_density=bwd_d, bwd_color=bwd_c,
        adam_grad_d=grad_d[:R, :R, :R], adam_m_d=m_d[:R, :R, :R], adam_v_d=v_d[:R, :R, :R],
        adam_lr=lr_d[:R, :R, :R], adam_grad_c=grad_c[:R, :R, :R], adam_m_c=m_c[:R, :R, :R],
        adam_v_c=v_c[:R, :R, :R], adam_hyper=np.array([stepsz, eps, b0, b1], np.float32),
        idx_rows=rows[:R, :R, :R], idx_den_rows=den_rows, idx_xyz=ixyz, idx_density=idx_den,
        idx_active_round=idx_act_round, **adam)
    for h in [gd, gg, hidx]:
        lib.nref_free_float(h)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
