"""The C-ABI library loads and exports every symbol include/pvdb.h declares;
argument validation runs before any device work (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pvdb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pvdb_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def built_lib():
    from plenvdb_gb300 import build
    path = build.build()
    return C.CDLL(path)


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for must in ("pvdb_grid_sample", "pvdb_grid_sample_backward", "pvdb_opt_step",
                 "pvdb_grid_tv_add_grad", "pvdb_march_forward", "pvdb_march_backward",
                 "pvdb_mlp_forward", "pvdb_train_step", "pvdb_renderer_render"):
        assert must in names


def test_every_declared_symbol_is_exported(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_the_header():
    from plenvdb_gb300 import _lib
    assert set(declared_functions()) <= set(_lib._SIGS)


def test_argument_errors_without_device(built_lib):
    from plenvdb_gb300 import _lib as L
    L.load()
    out = C.c_void_p()
    # channels must be 1 or a multiple of 3 (plenvdb.h:435, :530)
    rc = L.load().pvdb_grid_create(L.i32arr([8, 8, 8]), 2, 0.0, C.byref(out))
    assert rc == L.PVDB_ERR_ARG and "channels" in L.last_error()
    rc = L.load().pvdb_grid_create(L.i32arr([0, 8, 8]), 1, 0.0, C.byref(out))
    assert rc == L.PVDB_ERR_ARG and "resolution" in L.last_error()
    rc = L.load().pvdb_opt_step(None, 0, 0, None)
    assert rc == L.PVDB_ERR_ARG
    rc = L.load().pvdb_march_create(0, 10, C.byref(out))
    assert rc == L.PVDB_ERR_ARG
    with pytest.raises(L.PvdbError) as e:
        L.call("pvdb_grid_create", L.i32arr([8, 8, 8]), 4, 0.0, C.byref(out))
    assert e.value.code == L.PVDB_ERR_ARG


def test_lifecycle_argument_errors_without_device(built_lib):
    """The grid-lifecycle and ray entry points reject bad arguments before any
    device work (and empty inputs are no-ops)."""
    from plenvdb_gb300 import _lib as L
    lib = L.load()
    n = C.c_int64(-1)
    assert lib.pvdb_merge_count(None, 0, C.byref(n), None) == L.PVDB_OK and n.value == 0
    assert lib.pvdb_merge_count(None, 16, C.byref(n), None) == L.PVDB_ERR_ARG
    rc = lib.pvdb_merge_build(None, None, None, None, None, None, 1, 1, None)
    assert rc == L.PVDB_ERR_ARG and "grid" in L.last_error()
    keep = (C.c_uint8 * 4)()
    rc = lib.pvdb_compact_rows(keep, 4, None, None, 5, 4, C.byref(n), None)
    assert rc == L.PVDB_ERR_ARG and "four" in L.last_error()
    assert lib.pvdb_compact_rows(None, 0, None, None, 0, 0, C.byref(n), None) == L.PVDB_OK
    assert lib.pvdb_grid_resample(None, None, None) == L.PVDB_ERR_ARG
    shape = L.i32arr([4, 4, 4])
    box0, box1 = L.f32arr([-1] * 3), L.f32arr([1] * 3)
    rc = lib.pvdb_occupancy(None, 0, None, shape, box0, box1, -4.6, 0.5, 1e-3, None, None, None)
    assert rc == L.PVDB_ERR_ARG
    assert lib.pvdb_grid_maskout_near_cams(None, None, 1, box0, box1, 0.5, -100.0,
                                           None) == L.PVDB_ERR_ARG
    rc = lib.pvdb_count_views(None, None, 0, shape, box0, box1, 2.0, 0.01, 0, None, None, None)
    assert rc == L.PVDB_ERR_ARG
    K = L.f64arr([10, 0, 2, 0, 10, 2, 0, 0, 1])
    c2w = L.f32arr(np.eye(4).reshape(-1))
    rc = lib.pvdb_get_rays(4, 4, K, c2w, 0, 0, 0, 0, 3, None, None, None, None, None)
    assert rc == L.PVDB_ERR_ARG and "mode" in L.last_error()
    rc = lib.pvdb_get_rays(4, 4, K, c2w, 0, 0, 0, 0, 2, None, None, None, None, None)
    assert rc == L.PVDB_ERR_ARG and "jitter" in L.last_error()
    assert lib.pvdb_get_rays(0, 4, K, c2w, 0, 0, 0, 0, 0, None, None, None, None,
                             None) == L.PVDB_OK
    rc = lib.pvdb_rays_hit_mask(None, None, 1, box0, box1, 2.0, 0.01, None, shape, None, None)
    assert rc == L.PVDB_ERR_ARG


def test_samples_cap_bounds_the_bbox_chord(built_lib):
    from plenvdb_gb300 import _lib as L
    cap = L.load().pvdb_march_samples_cap(L.f32arr([-1.5] * 3), L.f32arr([1.5] * 3),
                                          0.5 * 3 / 160)
    import math
    assert cap >= math.ceil(math.sqrt(3) * 3 / (0.5 * 3 / 160))
    assert L.load().pvdb_march_samples_cap(L.f32arr([0] * 3), L.f32arr([1] * 3), 0.0) == 0
