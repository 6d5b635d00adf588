"""ctypes binding of ``libmeshoid_gb300.so`` (the C ABI in include/meshoid_gb300.h).

The library is the only compute path: there is no CPU fallback.  Loading fails
loudly when the library cannot be built or loaded, and every call checks the
returned status.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_f32 = ctypes.c_float
c_f64 = ctypes.c_double
c_vp = ctypes.c_void_p
c_sz = ctypes.c_size_t

MG_OK = 0
MG_ERR_ARG = 1
MG_ERR_CUDA = 2
MG_ERR_NOT_CONVERGED = 3
MG_ERR_UNSUPPORTED = 4
MG_ERR_NOALLOC_LIMIT = 5
MG_NOALLOC_MAX_QUERIES = 1 << 21
MG_MAX_K = 128
MG_MLP_IN = 54
MG_MLP_IN_PAD = 64
MG_MLP_HIDDEN = 64
MG_MLP_PARAM_COUNT = 64 * 64 + 64 + 64 * 64 + 64 + 64 + 1
MG_Q_UNRESOLVED = 1
MG_Q_BAND_FP64 = 2
MG_Q_SINGULAR = 4
MG_Q_FP64_SOLVE = 8
MG_Q_REFINED = 16
MG_BRICK_WORDS = 1028


class MgCells(ctypes.Structure):
    _fields_ = [
        ("n", c_i64),
        ("dim", c_i32),
        ("grid_level", c_i32),
        ("boxsize", c_f64),
        ("frame", c_vp),
        ("keys", c_vp),
        ("order", c_vp),
        ("rank", c_vp),
        ("pos_hi", c_vp),
        ("pos_lo", c_vp),
        ("pos64", c_vp),
        ("cell_start", c_vp),
        ("brick_of", c_vp),
        ("bricks", c_vp),
        ("brick_capacity", c_i32),
        ("brick_threshold", c_i32),
    ]


class MgSnapshot(ctypes.Structure):
    _fields_ = [
        ("n", c_i64),
        ("pos", c_vp),
        ("mass", c_vp),
        ("fields", c_vp),
        ("nf", c_i32),
        ("grid_level", c_i32),
        ("level_bias", c_i32),
        ("brick_threshold", c_i32),
        ("hsml", c_vp),
        ("grad", c_vp),
        ("map", c_vp),
        ("map_cx", c_f64),
        ("map_cy", c_f64),
        ("map_size", c_f64),
        ("map_res", c_i32),
        ("reserved", c_i32),
    ]


# name -> (restype, argtypes); mirrors include/meshoid_gb300.h
SIGNATURES = {
    "mg_status_string": (ctypes.c_char_p, [c_i32]),
    "mg_version": (c_i32, []),
    "mg_launch_count": (c_i64, []),
    "mg_default_grid_level": (c_i32, [c_i64]),
    "mg_build_cells_workspace_bytes": (c_sz, [c_i64, c_i32]),
    "mg_brick_capacity": (c_i32, [c_i64, c_i32, c_i32]),
    "mg_build_cells": (c_i32, [c_vp, ctypes.POINTER(MgCells), c_vp, c_sz, c_vp]),
    "mg_seed_plain": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_i32, c_vp, c_vp]),
    "mg_seed_features": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_i32, c_vp, c_vp, c_vp]),
    "mg_mlp_forward": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mg_mlp_train_step": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_f32, c_vp, c_vp, c_vp,
                                  c_vp, c_vp, c_vp, c_sz, c_vp]),
    "mg_mlp_train_workspace_bytes": (c_sz, [c_i64]),
    "mg_knn_hsml_workspace_bytes": (c_sz, [c_i64, c_i32]),
    "mg_knn_hsml": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_i32, c_vp, c_f32, c_i32, c_i32, c_vp,
                            c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "mg_neighbor_dist": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "mg_load_fields": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i32, c_vp, c_vp, c_vp]),
    "mg_load_fields3": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "mg_hsml_polish": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "mg_grad2_moments_bytes": (c_sz, [c_i64, c_i32]),
    "mg_grad2_moments": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_i32, c_f32,
                                 c_vp, c_sz, c_vp]),
    "mg_grad2_solve_workspace_bytes": (c_sz, [c_i64]),
    "mg_grad2_solve": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_i32, c_vp, c_sz,
                               c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "mg_grad_sweep_workspace_bytes": (c_sz, [c_i64]),
    "mg_grad_sweep": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_i32, c_i32, c_vp,
                              c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_f32, c_vp, c_sz, c_vp]),
    "mg_grad_sweep_noalloc": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_i32, c_i32,
                                      c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_f32, c_vp]),
    "mg_kernel_average": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_vp,
                                  c_i32, c_vp, c_vp, c_vp]),
    "mg_surface_density_workspace_bytes": (c_sz, [c_i64, c_i32]),
    "mg_surface_density": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_f64, c_f64, c_f64, c_i32, c_i32, c_vp, c_vp,
                                   c_sz, c_vp]),
    "mg_kernel_variance": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_i32, c_vp, c_vp, c_i32, c_vp, c_vp,
                                   c_vp]),
    "mg_hsml_solve": (c_i32, [c_vp, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp]),
    "mg_knn_set_group_pass": (c_i32, [c_i32]),
    "mg_knn_set_persistent_passes": (c_i32, [c_i32]),
    "mg_grad_set_refine": (c_i32, [c_i32]),
    "mg_kernel_weights": (c_i32, [c_vp, c_vp, c_i64, c_i32, c_vp, c_vp]),
    "mg_gradient_weights": (c_i32, [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_i64, c_f64, c_i32, c_i32, c_vp, c_vp,
                                    c_vp]),
    "mg_kde_1d_workspace_bytes": (c_sz, [c_i64]),
    "mg_kde_1d": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_sz, c_vp]),
    "mg_radtransfer_count": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_i32, c_f64, c_f64, c_f64, c_vp, c_vp]),
    "mg_radtransfer_workspace_bytes": (c_sz, [c_i64, c_i64, c_i32, c_i32]),
    "mg_radtransfer": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i32, c_i32, c_f64, c_f64, c_f64, c_f64, c_vp,
                               c_i64, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "mg_grid_density_count": (c_i32, [c_vp, c_vp, c_i64, c_f64, c_f64, c_f64, c_f64, c_i32, c_i32, c_vp, c_vp]),
    "mg_grid_density_workspace_bytes": (c_sz, [c_i64, c_i64, c_i32]),
    "mg_grid_density": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_f64, c_f64, c_f64, c_f64, c_i32, c_i32, c_vp, c_vp, c_i64,
                                c_vp, c_sz, c_vp]),
    "mg_ppz_cube": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_f64, c_f64, c_f64, c_f64, c_f64, c_i32, c_i32,
                            c_vp, c_vp]),
    "mg_weighted_interp3d": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, c_f64, c_f64, c_f64, c_f64, c_i32, c_vp, c_vp,
                                     c_vp, c_vp]),
    "mg_density": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "mg_batched_workspace_bytes": (c_sz, [ctypes.POINTER(MgSnapshot), c_i32, c_i32]),
    "mg_batched_run": (c_i32, [ctypes.POINTER(MgSnapshot), c_i32, c_i32, c_f32, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "mg_nn_query_workspace_bytes": (c_sz, [c_i64]),
    "mg_nn_query": (c_i32, [ctypes.POINTER(MgCells), c_vp, c_i64, c_vp, c_vp, c_sz, c_vp]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the shared library and bind the C ABI."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"meshoid_gb300: CUDA library not found at {path}; run meshoid_gb300.build.build()")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class MeshoidError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status != MG_OK:
        msg = load().mg_status_string(status).decode()
        raise MeshoidError(f"{what}: {msg} (status {status})")


def ptr(t):
    """Device pointer of a torch tensor (or None)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())
