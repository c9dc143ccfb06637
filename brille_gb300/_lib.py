"""Loader for the CUDA library (libbrx.so) through its C ABI.

There is no CPU fallback: if the library is missing or no GPU is present the
query path raises.
"""
from __future__ import annotations

import ctypes as C
import os

from ._abi import Atoms, Data, Geometry, LocateOut, MlpDims, SortCost, TrellisCells, TrellisIn

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbrx.so")

_lib = None


class BrxError(RuntimeError):
    """A non-OK status from the C ABI, carrying the library's message."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


def load(build_if_missing=True):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} has not been built; run brille_gb300.build.build()")
        from .build import build
        build()
    lib = C.CDLL(LIB_PATH)
    h = C.c_void_p
    lib.brx_create.argtypes = [C.POINTER(Geometry), C.c_int32, C.POINTER(h)]
    lib.brx_create.restype = C.c_int
    lib.brx_destroy.argtypes = [h]
    lib.brx_destroy.restype = None
    lib.brx_fill.argtypes = [h, C.POINTER(Data), C.POINTER(Data), C.c_int32]
    lib.brx_fill.restype = C.c_int
    lib.brx_set_permutations.argtypes = [h, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
    lib.brx_set_permutations.restype = C.c_int
    lib.brx_sort.argtypes = [h, C.c_int64, C.c_void_p, C.POINTER(SortCost), C.POINTER(SortCost), C.c_void_p]
    lib.brx_sort.restype = C.c_int
    lib.brx_get_permutations.argtypes = [h, C.c_int64, C.c_void_p, C.c_void_p]
    lib.brx_get_permutations.restype = C.c_int
    lib.brx_permutation_count.argtypes = [h]
    lib.brx_permutation_count.restype = C.c_int64
    for name in ("brx_ir_interpolate_at", "brx_interpolate_at"):
        f = getattr(lib, name)
        f.argtypes = [h, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        f.restype = C.c_int
    lib.brx_ir_interpolate_at_noalloc.argtypes = [h, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_uint32,
                                                  C.c_void_p]
    lib.brx_ir_interpolate_at_noalloc.restype = C.c_int
    lib.brx_locate.argtypes = [h, C.c_void_p, C.c_int64, C.c_int32, C.c_uint32, C.POINTER(LocateOut), C.c_void_p]
    lib.brx_locate.restype = C.c_int
    lib.brx_trellis_cells_build.argtypes = [C.POINTER(TrellisIn), C.c_int32, C.POINTER(TrellisCells)]
    lib.brx_trellis_cells_build.restype = C.c_int
    lib.brx_trellis_cells_free.argtypes = [C.POINTER(TrellisCells)]
    lib.brx_trellis_cells_free.restype = None
    lib.brx_sync.argtypes = [h, C.c_void_p]
    lib.brx_sync.restype = C.c_int
    lib.brx_last_error.argtypes = [h]
    lib.brx_last_error.restype = C.c_char_p
    lib.brx_launch_count.argtypes = [h]
    lib.brx_launch_count.restype = C.c_int64
    lib.brx_profile.argtypes = [h, C.c_int32]
    lib.brx_profile.restype = C.c_int
    lib.brx_stage_times.argtypes = [h, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.brx_stage_times.restype = C.c_int
    md = C.POINTER(MlpDims)
    vp = C.c_void_p
    lib.brx_mlp_param_count.argtypes = [md]
    lib.brx_mlp_param_count.restype = C.c_int64
    lib.brx_mlp_workspace_floats.argtypes = [md, C.c_int64]
    lib.brx_mlp_workspace_floats.restype = C.c_int64
    lib.brx_mlp_features.argtypes = [h, C.POINTER(LocateOut), C.c_int64, md, C.c_float, vp, vp, vp]
    lib.brx_mlp_features.restype = C.c_int
    lib.brx_mlp_train_step.argtypes = [md, vp, vp, vp, vp, C.c_int32, C.c_float, vp, vp, C.c_int64, vp, vp, vp]
    lib.brx_mlp_train_step.restype = C.c_int
    lib.brx_mlp_forward.argtypes = [md, vp, vp, C.c_int64, vp, vp, vp]
    lib.brx_mlp_forward.restype = C.c_int
    lib.brx_set_residual_model.argtypes = [h, md, vp, C.c_float, C.c_float, C.c_float]
    lib.brx_set_residual_model.restype = C.c_int
    lib.brx_set_atoms.argtypes = [h, C.POINTER(Atoms)]
    lib.brx_set_atoms.restype = C.c_int
    lib.brx_ir_structure_factor.argtypes = [h, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    lib.brx_ir_structure_factor.restype = C.c_int
    bp = C.c_void_p
    lib.brx_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_int64), C.c_int32, C.c_uint32,
                                     C.POINTER(C.c_void_p)]
    lib.brx_batch_create.restype = C.c_int
    lib.brx_batch_destroy.argtypes = [bp]
    lib.brx_batch_destroy.restype = None
    lib.brx_batch_set_io.argtypes = [bp, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    lib.brx_batch_set_io.restype = C.c_int
    for name in ("brx_batch_run", "brx_batch_capture", "brx_batch_launch"):
        getattr(lib, name).argtypes = [bp, C.c_void_p]
        getattr(lib, name).restype = C.c_int
    lib.brx_batch_sync.argtypes = [bp, C.c_void_p, C.POINTER(C.c_int32)]
    lib.brx_batch_sync.restype = C.c_int
    lib.brx_batch_tune.argtypes = [bp, C.c_void_p, C.c_int32]
    lib.brx_batch_tune.restype = C.c_int
    lib.brx_batch_config.argtypes = [bp, C.POINTER(C.c_int32), C.c_int32]
    lib.brx_batch_config.restype = C.c_int
    lib.brx_batch_set_config.argtypes = [bp, C.POINTER(C.c_int32), C.c_int32]
    lib.brx_batch_set_config.restype = C.c_int
    lib.brx_batch_launch_count.argtypes = [bp]
    lib.brx_batch_launch_count.restype = C.c_int64
    lib.brx_batch_last_error.argtypes = [bp]
    lib.brx_batch_last_error.restype = C.c_char_p
    lib.brx_tune.argtypes = [h, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32]
    lib.brx_tune.restype = C.c_int
    lib.brx_tuning.argtypes = [h, C.POINTER(C.c_int32), C.c_int32]
    lib.brx_tuning.restype = C.c_int
    lib.brx_set_tuning.argtypes = [h, C.POINTER(C.c_int32), C.c_int32]
    lib.brx_set_tuning.restype = C.c_int
    lib.brx_abi_version.argtypes = []
    lib.brx_abi_version.restype = C.c_int32
    _lib = lib
    return lib


def check(status, handle=None):
    if status != 0:
        msg = load().brx_last_error(handle).decode() if handle else f"status {status}"
        raise BrxError(status, msg)
