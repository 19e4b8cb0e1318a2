"""The C-ABI library loads and exports every symbol include/pvdb.h declares;
argument validation runs before any device work (no GPU needed)."""
import ctypes as C
import os
import re

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


def test_samples_cap_bounds_the_bbox_chord(built_lib):
    from plenvdb_gb300 import _lib as L
    cap = L.load().pvdb_march_samples_cap(L.f32arr([-1.5] * 3), L.f32arr([1.5] * 3),
                                          0.5 * 3 / 160)
    import math
    assert cap >= math.ceil(math.sqrt(3) * 3 / (0.5 * 3 / 160))
    assert L.load().pvdb_march_samples_cap(L.f32arr([0] * 3), L.f32arr([1] * 3), 0.0) == 0
