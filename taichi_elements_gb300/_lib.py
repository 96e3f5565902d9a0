"""ctypes binding of libmpm_gb300.so (declared in include/mpm_gb300.h).

Structures mirror the C header field for field.  Loading fails loudly when
the library is missing or was built for another ABI: the engine has no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import build as _build

ABI_VERSION = 6
NROWS = 28
QROWS = 21  # packed rows of quant=True (MPM_QROWS)
MAX_COLLIDERS = 16

STATUS_OUT_OF_GRID = 1
STATUS_NONFINITE = 2
STATUS_TABLE_OVERFLOW = 4
STATUS_UNSUPPORTED = 8
STATUS_TIMEOUT = 16

# Row indices of the particle-state buffer.
ROW_X, ROW_V, ROW_C, ROW_F, ROW_JP, ROW_MAT, ROW_ID, ROW_EP = 0, 3, 6, 15, 24, 25, 26, 27

# Post-process record kinds.
KIND_SURFACE, KIND_SPHERE, KIND_BOX = 0, 1, 2

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "ABI version mismatch", -4: "capacity exceeded"}


class MpmCollider(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("surface", ctypes.c_int32),
        ("point", ctypes.c_float * 3),
        ("normal", ctypes.c_float * 3),
        ("radius", ctypes.c_float),
        ("friction", ctypes.c_float),
    ]


class MpmParams(ctypes.Structure):
    _fields_ = [
        ("version", ctypes.c_int32),
        ("res", ctypes.c_int32 * 3),
        ("padding", ctypes.c_int32),
        ("unbounded", ctypes.c_int32),
        ("grid_size", ctypes.c_int32),
        ("n_colliders", ctypes.c_int32),
        ("win_lo", ctypes.c_int32 * 3),
        ("win_nb", ctypes.c_int32 * 3),
        ("has_Ep", ctypes.c_int32),
        ("chunk", ctypes.c_int32),
        ("plasticity", ctypes.c_int32),
        ("quant", ctypes.c_int32),
        ("occupancy", ctypes.c_int32),
        ("dx", ctypes.c_float),
        ("inv_dx", ctypes.c_float),
        ("p_vol", ctypes.c_float),
        ("p_mass", ctypes.c_float),
        ("mu0", ctypes.c_float),
        ("la0", ctypes.c_float),
        ("nu", ctypes.c_float),
        ("alpha", ctypes.c_float),
        ("water_density", ctypes.c_float),
        ("gravity", ctypes.c_float * 3),
        ("stress_k", ctypes.c_float),
        ("sand_k", ctypes.c_float),
        ("v_clamp_k", ctypes.c_float),
        ("n_scenes", ctypes.c_int32),
        ("slot_nb", ctypes.c_int32 * 3),
        ("slots", ctypes.c_int32 * 3),
        ("dt", ctypes.c_float),
        ("colliders", MpmCollider * MAX_COLLIDERS),
    ]


class MpmViews(ctypes.Structure):
    _fields_ = [
        ("counters", ctypes.c_void_p),
        ("pblocks", ctypes.c_void_p),
        ("gblocks", ctypes.c_void_p),
        ("pblock_count", ctypes.c_void_p),
        ("pblock_start", ctypes.c_void_p),
        ("pid", ctypes.c_void_p),
        ("cellkey", ctypes.c_void_p),
        ("grid_mom", ctypes.c_void_p),
        ("grid_vel", ctypes.c_void_p),
    ]


# Every exported symbol with its argument types (all return int).
_P = ctypes.POINTER(MpmParams)
_v = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_f = ctypes.c_float
SIGNATURES = {
    "mpm_abi_version": [],
    "mpm_workspace_bytes": [_P, _i64, ctypes.POINTER(ctypes.c_size_t)],
    "mpm_workspace_init": [_P, _v, _i64, _v],
    "mpm_bin_count": [_P, _v, _i64, _v, _i64, _i64, _v],
    "mpm_bin_finalize": [_P, _v, _i64, _i64, _v],
    "mpm_p2g": [_P, _v, _i64, _i64, _v, _v, _f, _v],
    "mpm_grid_update": [_P, _v, _i64, _f, _v],
    "mpm_g2p": [_P, _v, _i64, _i64, _v, _f, _v, _v],
    "mpm_substep": [_P, _v, _i64, _i64, _v, _v, _f, _v, _v],
    "mpm_frame": [_P, _v, _i64, _i64, _v, _v, _f, _i32, _i32, _v, _v, _v, _v],
    "mpm_g2p2g_frame": [_P, _v, _i64, _i64, _v, _v, _f, _i32, _i32, _i64, _v, _v, _v, _v],
    "mpm_batch_frame": [_P, _v, _v, _i64, _i64, _v, _v, _i32, _i32, _v, _v, _v, _v],
    "mpm_g2p2g_substep": [_P, _v, _i64, _i64, _v, _v, _f, _i64, _i32, _v, _v],
    "mpm_substep_noalloc": [_P, _i64, _i64, _v, _v, _f, _v, _v],
    "mpm_batch_bin_count": [_P, _v, _v, _i64, _v, _i64, _i64, _v],
    "mpm_grid_snapshot": [_P, _v, _i64, _v, _v],
    "mpm_g2p_bin_into": [_P, _v, _v, _i64, _i64, _v, _f, _v, _v],
    "mpm_grad_reorder": [_v, _i64, _i64, _i32, _v, _v, _i32, _v],
    "mpm_particle_ranges": [_v, _i64, _i64, _v, _v, _v],
    "mpm_quantize_particles": [_v, _i64, _i64, _v, _v, _v],
    "mpm_unpack_colors": [_v, _i64, _v, _v],
    "mpm_render_scene_bytes": [],
    "mpm_render_cell_count": [_v, _v, _v, _i64, _v, _v],
    "mpm_render_cell_fill": [_v, _v, _v, _i64, _v, _v, _i64, _v, _v],
    "mpm_render_occupancy": [_v, _i64, _v, _v],
    "mpm_render_samples": [_v, _v, _v, _v, _v, _v, _v, _v, _i32, _i32, _v, _v],
    "mpm_render_tonemap": [_i32, _i32, _v, _f, _f, _f, _f, _f, _i32, _v, _v],
    "mpm_render_first_hits": [_v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _i64, _f, _v, _v],
    "mpm_voxelize": [_v, _i64, _i32, _i32, _i32, ctypes.c_double, _i32, _v, _v],
    "mpm_voxel_seed_count": [_v, _i32, _i32, _i32, _i32, _i32, _i32, _i32, ctypes.c_uint64, _v, _v],
    "mpm_voxel_seed_emit": [_v, _i32, _i32, _i32, _i32, _i32, _i32, _i32, ctypes.c_uint64, _f, _f, _f, _f, _v,
                            _i64, _v, _v],
    "mpm_g2p_adj": [_P, _v, _i64, _i64, _v, _f, _v, _v, _v, _i32, _v],
    "mpm_grid_adj": [_P, _v, _i64, _v, _v, _f, _v],
    "mpm_p2g_adj": [_P, _v, _i64, _i64, _v, _f, _v, _v, _v, _v, _i32, _v],
    "mpm_batch_substep": [_P, _v, _v, _i64, _i64, _v, _v, _v, _v],
    "mpm_gather_rows": [_v, _i64, _i64, _i32, _i32, _v, _v],
    "mpm_quant_pack": [_v, _i64, _i64, _v, _i64, _i64, _v, _v],
    "mpm_quant_unpack": [_v, _i64, _i64, _i64, _v, _i64, _v],
    "mpm_status_ptr": [_P, _v, _i64, ctypes.POINTER(ctypes.c_void_p)],
    "mpm_max_grid_velocity": [_P, _v, _i64, _v, _v],
    "mpm_constitutive_eval": [_P, _i64, _v, _v, _v, _v, _v, _f, _v],
    "mpm_views": [_P, _v, _i64, ctypes.POINTER(MpmViews)],
}

_lock = threading.Lock()
_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the engine library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.library_path()
        if build_if_missing:
            path = _build.build_library()
        if not Path(path).exists():
            raise RuntimeError(f"GB300 engine library not found at {path}; run build() first")
        lib = ctypes.CDLL(str(path))
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = ctypes.c_int
        if lib.mpm_abi_version() != ABI_VERSION:
            raise RuntimeError("libmpm_gb300.so ABI version mismatch")
        _lib = lib
        return lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed: {ERRORS.get(rc, rc)}")
