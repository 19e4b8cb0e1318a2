"""ctypes binding of libpvdb.so (include/pvdb.h).

The library is loaded from this package directory; importing a module that
needs it raises ImportError when it has not been built (run
``python -m plenvdb_gb300.build`` or ``__graft_entry__.build()``). There is no
CPU fallback: every call goes to the CUDA library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpvdb.so")

PVDB_OK = 0
PVDB_ERR_ARG = 1
PVDB_ERR_CUDA = 2
PVDB_ERR_TIMEOUT = 3
PVDB_ERR_NOMEM = 4
PVDB_ERR_STATE = 5
PVDB_ERR_IO = 6

MEM_HOST = 0
MEM_DEVICE = 1
WHICH_DATA = 0
WHICH_GRAD = 1

_ERR_NAMES = {1: "PVDB_ERR_ARG", 2: "PVDB_ERR_CUDA", 3: "PVDB_ERR_TIMEOUT",
              4: "PVDB_ERR_NOMEM", 5: "PVDB_ERR_STATE", 6: "PVDB_ERR_IO"}


class PvdbError(RuntimeError):
    """A libpvdb call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
f32 = C.c_float
P_i32 = C.POINTER(C.c_int32)
P_f32 = C.POINTER(C.c_float)


class MarchParams(C.Structure):
    _fields_ = [("xyz_min", f32 * 3), ("xyz_max", f32 * 3), ("near_", f32), ("far_", f32),
                ("stepdist", f32), ("act_shift", f32), ("interval", f32),
                ("fast_color_thres", f32), ("t_stop", f32), ("bg", f32)]


class MarchViews(C.Structure):
    _fields_ = [("alphainv_last", vp), ("n_kept", vp), ("n_color", vp), ("color_offset", vp),
                ("k0", vp), ("weight", vp), ("alpha", vp), ("ray_id", vp), ("step_id", vp),
                ("totals", vp), ("rows_capacity", i64)]


class MlpWeights(C.Structure):
    _fields_ = [("w0", vp), ("b0", vp), ("w1", vp), ("b1", vp), ("w2", vp), ("b2", vp),
                ("c0", i32), ("pe", i32), ("width", i32)]


class MlpGrads(C.Structure):
    _fields_ = [("w0", vp), ("b0", vp), ("w1", vp), ("b1", vp), ("w2", vp), ("b2", vp)]


class TrainConfig(C.Structure):
    _fields_ = [("march", MarchParams), ("weight_main", f32), ("weight_entropy_last", f32),
                ("weight_rgbper", f32), ("tv_weight_density", f32), ("tv_weight_k0", f32),
                ("tv_dense_mode", i32), ("lr_decay_factor", f32), ("rgbnet_lr", f32),
                ("rgbnet_beta1", f32), ("rgbnet_beta2", f32), ("rgbnet_eps", f32),
                ("precision", i32), ("use_graph", i32), ("tv_in_place", i32)]


class RgbnetState(C.Structure):
    _fields_ = [("params", vp), ("grads", vp), ("exp_avg", vp), ("exp_avg_sq", vp),
                ("step", P_i32), ("lr", P_f32), ("c0", i32), ("pe", i32), ("width", i32)]


# name -> (restype, argtypes)
_SIGS = {
    "pvdb_version": (C.c_char_p, []),
    "pvdb_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "pvdb_debug_fail_next_allocs": (C.c_int, [C.c_int]),
    "pvdb_debug_wait_limit": (C.c_int, [C.c_uint32, i32]),
    "pvdb_debug_k0_blocks": (C.c_int, [C.c_int]),
    "pvdb_grid_touched_leaves": (C.c_int, [vp, C.POINTER(i64), vp]),
    "pvdb_profile_begin": (C.c_int, [i32]),
    "pvdb_profile_end": (C.c_int, [P_f32, i32, P_i32]),
    "pvdb_launch_count": (C.c_uint64, []),
    "pvdb_grid_create": (C.c_int, [P_i32, i32, f32, C.POINTER(vp)]),
    "pvdb_grid_create_from_mask": (C.c_int, [P_i32, i32, f32, vp, i32, C.POINTER(vp)]),
    "pvdb_grid_create_like": (C.c_int, [vp, i32, f32, C.POINTER(vp)]),
    "pvdb_grid_destroy": (C.c_int, [vp]),
    "pvdb_grid_get_info": (C.c_int, [vp, P_i32, P_i32, P_i32, C.POINTER(i64), P_f32]),
    "pvdb_grid_set_reso": (C.c_int, [vp, i32, i32, i32]),
    "pvdb_grid_copy_from_dense": (C.c_int, [vp, i32, vp, i64, i32, vp]),
    "pvdb_grid_copy_to_dense": (C.c_int, [vp, i32, vp, i64, i32, vp]),
    "pvdb_grid_set_values_by_mask": (C.c_int, [vp, vp, i64, f32, i32, vp]),
    "pvdb_grid_sample": (C.c_int, [vp, vp, vp, vp, i64, vp, i32, vp]),
    "pvdb_grid_sample_backward": (C.c_int, [vp, vp, vp, vp, vp, i64, i32, vp]),
    "pvdb_grid_sample_backward_noalloc": (C.c_int, [vp, vp, vp, vp, vp, i64, vp]),
    "pvdb_grid_lookup": (C.c_int, [vp, vp, vp, vp, i64, vp, vp, i32, vp]),
    "pvdb_grid_tv_add_grad": (C.c_int, [vp, f32, f32, f32, i32, i32, vp]),
    "pvdb_grid_zero_grad": (C.c_int, [vp, vp]),
    "pvdb_grid_device_views": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                         C.POINTER(vp), C.POINTER(vp), P_i32]),
    "pvdb_grid_mark_written": (C.c_int, [vp, i32]),
    "pvdb_grid_save": (C.c_int, [vp, C.c_char_p]),
    "pvdb_grid_load": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "pvdb_opt_create": (C.c_int, [vp, f32, f32, f32, f32, C.POINTER(vp)]),
    "pvdb_opt_destroy": (C.c_int, [vp]),
    "pvdb_opt_step": (C.c_int, [vp, i32, i32, vp]),
    "pvdb_opt_zero_grad": (C.c_int, [vp, vp]),
    "pvdb_opt_set_grad": (C.c_int, [vp, vp, i64, i32, vp]),
    "pvdb_opt_set_pervoxel_lr": (C.c_int, [vp, vp, i64, i32, vp]),
    "pvdb_opt_update_lr": (C.c_int, [vp, f32]),
    "pvdb_opt_get_scalars": (C.c_int, [vp, P_i32, P_f32, P_f32, P_f32, P_f32]),
    "pvdb_opt_set_scalars": (C.c_int, [vp, i32, f32, f32, f32, f32]),
    "pvdb_opt_moments": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "pvdb_adam_dense": (C.c_int, [vp, vp, vp, vp, vp, i64, i32, f32, f32, f32, f32, i32, vp]),
    "pvdb_raw2alpha": (C.c_int, [vp, i64, f32, f32, vp, vp, vp]),
    "pvdb_raw2alpha_backward": (C.c_int, [vp, vp, i64, f32, vp, vp]),
    "pvdb_alpha2weight": (C.c_int, [vp, vp, i64, i32, vp, vp, vp, vp, vp, vp]),
    "pvdb_alpha2weight_backward": (C.c_int, [vp, vp, vp, vp, vp, vp, i32, vp, vp, i64, vp, vp]),
    "pvdb_ray_count_samples": (C.c_int, [vp, vp, i32, P_f32, P_f32, f32, f32, f32, vp, vp, vp,
                                         vp]),
    "pvdb_ray_sample_points": (C.c_int, [vp, vp, i32, P_f32, P_f32, f32, vp, vp, i64, vp, vp,
                                         vp, vp, vp]),
    "pvdb_maskcache_lookup": (C.c_int, [vp, P_i32, vp, i64, P_f32, P_f32, vp, vp]),
    "pvdb_march_create": (C.c_int, [i32, i32, C.POINTER(vp)]),
    "pvdb_march_destroy": (C.c_int, [vp]),
    "pvdb_march_set_leaf_staging": (C.c_int, [vp, i32]),
    "pvdb_march_samples_cap": (i32, [P_f32, P_f32, f32]),
    "pvdb_march_forward": (C.c_int, [vp, vp, vp, vp, vp, i32, C.POINTER(MarchParams), vp, P_i32,
                                     vp]),
    "pvdb_march_views": (C.c_int, [vp, C.POINTER(MarchViews)]),
    "pvdb_march_totals": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), vp]),
    "pvdb_march_stats": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), vp]),
    "pvdb_march_adam_counts": (C.c_int, [vp, C.POINTER(i64), vp]),
    "pvdb_march_backward": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "pvdb_composite_forward": (C.c_int, [vp, vp, f32, vp, i32, vp]),
    "pvdb_composite_backward": (C.c_int, [vp, vp, vp, f32, vp, vp, vp, i32, vp]),
    "pvdb_mlp_forward": (C.c_int, [vp, C.POINTER(MlpWeights), vp, vp, vp, i32, vp]),
    "pvdb_mlp_backward": (C.c_int, [vp, C.POINTER(MlpWeights), vp, vp, vp, vp,
                                    C.POINTER(MlpGrads), vp, i32, vp]),
    "pvdb_train_step": (C.c_int, [vp, vp, vp, C.POINTER(RgbnetState), vp, vp, vp, vp, i32,
                                  C.POINTER(TrainConfig), vp, vp]),
    "pvdb_renderer_create": (C.c_int, [i32, i32, i32, i32, C.POINTER(vp)]),
    "pvdb_renderer_destroy": (C.c_int, [vp]),
    "pvdb_renderer_load_data": (C.c_int, [vp, P_i32, vp, vp, vp, i64, i32, i32]),
    "pvdb_renderer_load_params": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "pvdb_renderer_set_scene": (C.c_int, [vp, P_i32, P_f32, P_f32, P_f32]),
    "pvdb_renderer_set_kwargs": (C.c_int, [vp, f32, f32, f32, f32, f32, f32, f32, i32, i32, i32,
                                           f32]),
    "pvdb_renderer_input_c2w": (C.c_int, [vp, vp, i32, vp]),
    "pvdb_renderer_render": (C.c_int, [vp, i32, vp]),
    "pvdb_renderer_output": (C.c_int, [vp, vp, i32, vp]),
    "pvdb_renderer_views": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "pvdb_merge_count": (C.c_int, [vp, i64, C.POINTER(i64), vp]),
    "pvdb_merge_build": (C.c_int, [vp, vp, vp, vp, vp, vp, i64, i32, vp]),
    "pvdb_compact_rows": (C.c_int, [vp, i64, vp, vp, i32, i64, C.POINTER(i64), vp]),
    "pvdb_grid_resample": (C.c_int, [vp, vp, vp]),
    "pvdb_occupancy": (C.c_int, [vp, i32, vp, P_i32, P_f32, P_f32, f32, f32, f32, vp, P_i32,
                                 vp]),
    "pvdb_grid_maskout_near_cams": (C.c_int, [vp, vp, i32, P_f32, P_f32, f32, f32, vp]),
    "pvdb_count_views": (C.c_int, [vp, vp, i64, P_i32, P_f32, P_f32, f32, f32, i32, vp, vp, vp]),
    "pvdb_get_rays": (C.c_int, [i32, i32, C.POINTER(C.c_double), P_f32, i32, i32, i32, i32, i32,
                                vp, vp, vp, vp, vp]),
    "pvdb_rays_hit_mask": (C.c_int, [vp, vp, i64, P_f32, P_f32, f32, f32, vp, P_i32, vp, vp]),
}

_lib = None


def load(path: str | None = None):
    """Load libpvdb.so once and attach the signatures. Raises ImportError if missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"libpvdb.so not built at {path}; run plenvdb_gb300/build.py")
    lib = C.CDLL(path, mode=C.RTLD_GLOBAL)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols(path: str | None = None) -> set[str]:
    lib = C.CDLL(path or LIB_PATH)
    return {n for n in _SIGS if hasattr(lib, n)}


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().pvdb_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int):
    if rc != PVDB_OK:
        raise PvdbError(rc, last_error())


def call(name: str, *args):
    check(getattr(load(), name)(*args))


# ---------------------------------------------------------------- pointers
def ptr(x) -> int | None:
    """Raw address of a numpy array or torch tensor (None passes NULL)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


def i32arr(vals) -> C.Array:
    return (C.c_int32 * len(vals))(*[int(v) for v in vals])


def f32arr(vals) -> C.Array:
    return (C.c_float * len(vals))(*[float(v) for v in vals])


def f64arr(vals) -> C.Array:
    return (C.c_double * len(vals))(*[float(v) for v in vals])


def ptrarr(ptrs) -> C.Array:
    return (C.c_void_p * max(len(ptrs), 1))(*ptrs)


def is_cuda(x) -> bool:
    return not isinstance(x, np.ndarray) and getattr(x, "is_cuda", False)


def stream_of(x=None) -> int | None:
    """The current torch CUDA stream handle (None = legacy default stream)."""
    try:
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            return torch.cuda.current_stream().cuda_stream
    except Exception:
        pass
    return None
