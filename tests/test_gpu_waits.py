"""Bounded device-side waits report PVDB_ERR_TIMEOUT and leave the context
usable. Each test makes a look-back wait run out on purpose through the
library's test hook (pvdb_debug_wait_limit: a short spin limit, and the first
publisher of the look-back chain withholds its count, so the waits behind it
see a flag that nothing sets). Every wait is bounded; a wait that gives up
keeps every access in bounds (its prefix is at most the true one) and the
kernels after it skip their work. Then the hook is reset and the same call is
checked against an undisturbed run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def hold(lib):
    from plenvdb_gb300 import _lib as L
    L.call("pvdb_debug_wait_limit", 4096, 1)
    yield L
    L.call("pvdb_debug_wait_limit", 0, 0)


def _points(rng, n, reso):
    import torch
    xyz = torch.from_numpy(rng.uniform(-0.5, np.array(reso) + 0.5, (n, 3)).astype(np.float32))
    xyz = xyz.cuda()
    return [xyz[:, q].contiguous() for q in range(3)]


@pytest.mark.parametrize("entry", ["pvdb_grid_sample_backward", "pvdb_grid_sample_backward_noalloc"])
def test_grid_backward_sort_wait_reports_timeout(hold, entry):
    import torch
    from plenvdb_gb300 import DensityVDB
    L = hold
    rng = np.random.default_rng(3)
    reso = [40, 40, 40]
    n = 8192  # 65536 (slot, id) pairs: 64 sort tiles, so the look-back waits
    xs, ys, zs = _points(rng, n, reso)
    g = torch.from_numpy(rng.normal(0, 1, n).astype(np.float32)).cuda()

    def run(grid):
        args = [grid.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs), L.ptr(g), n]
        if entry == "pvdb_grid_sample_backward":
            args.append(L.MEM_DEVICE)
        return getattr(L.load(), entry)(*args, L.stream_of())

    a = DensityVDB(reso, 1)
    rc = run(a)
    assert rc == L.PVDB_ERR_TIMEOUT, (rc, L.last_error())
    assert "timed out" in L.last_error()
    # the reduction after the sort skipped its work: the gradient is unchanged
    assert not np.any(a.get_dense_grid(which=L.WHICH_GRAD))
    # the context is usable and, with the hook reset, the call is exact again
    L.call("pvdb_debug_wait_limit", 0, 0)
    b = DensityVDB(reso, 1)
    assert run(a) == L.PVDB_OK and run(b) == L.PVDB_OK
    np.testing.assert_array_equal(a.get_dense_grid(which=L.WHICH_GRAD),
                                  b.get_dense_grid(which=L.WHICH_GRAD))
    assert np.any(b.get_dense_grid(which=L.WHICH_GRAD))


def test_march_ray_offset_wait_reports_timeout(hold):
    import torch
    from plenvdb_gb300.march import MarchWorkspace, march_params
    from plenvdb_gb300.scene import CameraConfig, SceneConfig, build_grids, random_rays
    L = hold
    scfg = SceneConfig(reso=40, n_ellipsoids=4, seed=3)
    dg, _ = build_grids(scfg)
    R = 512
    ro, rd, _ = random_rays(CameraConfig(), R, 4, seed=2)
    tro, trd = torch.from_numpy(ro).cuda(), torch.from_numpy(rd).cuda()
    lo, hi, step = [-1.5] * 3, [1.5] * 3, 0.5 * 3.0 / 40
    p = march_params(lo, hi, 2.0, step, -4.6, 0.5, 1e-4)
    ws = MarchWorkspace(R, lo, hi, step)

    def forward():
        L.call("pvdb_march_forward", ws.h, dg.handle, None, L.ptr(tro), L.ptr(trd), R,
               C.byref(p), None, None, L.stream_of())
        tk, tr = C.c_int64(), C.c_int64()
        rc = L.load().pvdb_march_totals(ws.h, C.byref(tk), C.byref(tr), L.stream_of())
        return rc, tk.value, tr.value

    rc, _, _ = forward()
    assert rc == L.PVDB_ERR_TIMEOUT, (rc, L.last_error())
    assert "look-back" in L.last_error()
    L.call("pvdb_debug_wait_limit", 0, 0)
    rc1, k1, r1 = forward()
    rc2, k2, r2 = forward()
    assert rc1 == rc2 == L.PVDB_OK
    assert (k1, r1) == (k2, r2) and k1 > 0 and r1 > 0


def test_rgbnet_backward_mma_wait_reports_timeout(lib):
    """The tensor-core rgbnet backward with the hook set: its MMA issuer
    withholds every MMA, the epilogue warps' waits on the MMA barrier run out,
    the CTAs release TMEM and write zero partials, and the march workspace
    reports PVDB_ERR_TIMEOUT. A clean run afterwards is bitwise equal to a
    run that never saw the hook. (The hook is set around the backward only:
    the march forward's look-back would otherwise give up first.)"""
    import torch
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300.march import MarchSample, MarchWorkspace, RgbNetFn, march_params
    from plenvdb_gb300.scene import (CameraConfig, SceneConfig, build_grids, random_rays,
                                     rgbnet_init)
    scfg = SceneConfig(reso=40, n_ellipsoids=4, seed=3)
    dg, kg = build_grids(scfg)
    R = 512
    ro, rd, vd = random_rays(CameraConfig(), R, 4, seed=2)
    tro, trd, tvd = (torch.from_numpy(a).cuda() for a in (ro, rd, vd))
    lo, hi, step = [-1.5] * 3, [1.5] * 3, 0.5 * 3.0 / 40
    p = march_params(lo, hi, 2.0, step, -4.6, 0.5, 1e-4)
    ws = MarchWorkspace(R, lo, hi, step)
    dummy = torch.zeros(1, device="cuda", requires_grad=True)

    def grads(held):
        w, last, k0, rid = MarchSample.apply(dummy, ws, dg, kg, tro, trd, p)
        params = [t.cuda().requires_grad_() for t in rgbnet_init(seed=3)]
        k0r = k0.detach().clone().requires_grad_()
        rgb = RgbNetFn.apply(k0r, tvd, ws, 4, 1, *params)
        assert rgb.shape[0] > 128  # more than one 128-row tile
        if held:
            L.call("pvdb_debug_wait_limit", 4096, 1)
        try:
            rgb.backward(torch.ones_like(rgb))
            torch.cuda.synchronize()
        finally:
            L.call("pvdb_debug_wait_limit", 0, 0)
        tk, tr = C.c_int64(), C.c_int64()
        rc = L.load().pvdb_march_totals(ws.h, C.byref(tk), C.byref(tr), L.stream_of())
        if held:
            assert rc == L.PVDB_ERR_TIMEOUT, (rc, L.last_error())
            assert "MMA" in L.last_error()
            return None
        assert rc == L.PVDB_OK, L.last_error()
        return [t.grad.cpu().numpy() for t in params] + [k0r.grad.cpu().numpy()]

    grads(held=True)
    a = grads(held=False)
    b = grads(held=False)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert np.abs(a[0]).sum() > 0
